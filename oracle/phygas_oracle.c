/* phygas_oracle.c -- CPU oracle for the Phygas orbit hot paths.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker, not the product: only the tests, the smoke check and the CPU-baseline leg of bench.py
 * load it (as oracle/_build/libphygas_oracle.so).  It restates, operation by operation and in the same
 * floating-point order, the reference's CPU algorithm for the two paths the GPU library implements:
 *   the linear star x cluster screen  (reference src/phygas.c:251-450)
 *   the ph_pair clone Monte Carlo     (reference src/phygas.c:146-249)
 * together with what feeds them: the Allen & Santillan (1991) force law (src/potential.c:28-101), the astrometry ->
 * Galactocentric transform (src/coords.c:77-131), splitmix64 + Box-Muller (src/montecarlo.h:26-41,
 * src/montecarlo.c:4-17), the draws with radial-velocity priors (src/phygas.c:21-82), tracks and the prefilter
 * (src/phygas.c:84-168), ph_seed (src/phygas.c:452-458) and the file readers (src/phygas.c:460-506).
 *
 * The arithmetic must be evaluated exactly as the reference evaluates it (same association, same constants,
 * no contraction of a*b+c: build with -std=c99 -ffp-contract=off) because the oracle is pinned bit for bit against
 * the reference compiled from its own sources (oracle/Makefile -> oracle/_ref) and against the reference's published
 * row hashes.  Where a formula below looks like the reference's, that is why: it is the same computation.
 *
 * It exports the reference's own C API (include/phygas.h), so one test harness drives the reference build, this
 * oracle and the GPU library through identical calls.
 */
#include "phygas.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---- units and parameters (reference src/units.h:14,27-28; src/potential.c:34-45; src/coords.c:63-70) ---- */
#define KMS_PER_KPCMYR 977.7922216807892
#define G_KPC (4.30091e-6 / (KMS_PER_KPCMYR * KMS_PER_KPCMYR))
#define MGAL 2.325e7
#define PI_LIT 3.14159265358979323846
#define DEG_TO_RAD (PI_LIT / 180.0)
#define AU_PER_YR_KMS (1.495978707e8 / 3.15576e7)

const MilkyWayParams milkyway_potential_default = {
    G_KPC * (606.0 * MGAL), 0.3873,
    G_KPC * (3690.0 * MGAL), 5.3178, 0.2500,
    G_KPC * (4615.0 * MGAL), 12.0, 100.0, 2.02,
};
const SolarParams solar_params_default = {8.122, 0.0208, 229.0, 11.1, 12.24, 7.25};

/* ICRS -> Galactic rotation (Hipparcos definition; reference src/coords.c:27-31) */
static const double ROT[3][3] = {
    {-0.0548755604162154, -0.8734370902348850, -0.4838350155487132},
    {0.4941094278755837, -0.4448296299600112, 0.7469822444972189},
    {-0.8676661490190047, -0.1980763734312015, 0.4559837761750669},
};

static Vec3 vmk(double x, double y, double z) { Vec3 v; v.x = x; v.y = y; v.z = z; return v; }
static Vec3 vplus(Vec3 a, Vec3 b) { return vmk(a.x + b.x, a.y + b.y, a.z + b.z); }
static Vec3 vminus(Vec3 a, Vec3 b) { return vmk(a.x - b.x, a.y - b.y, a.z - b.z); }
static Vec3 vtimes(Vec3 a, double s) { return vmk(a.x * s, a.y * s, a.z * s); }
static double vdot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static double vlen(Vec3 a) { return sqrt(vdot(a, a)); }

/* ---- force law (reference src/potential.c:53-101) ---------------------------------------------------------- */
static double halo_mass(const MilkyWayParams *p, double r) {
    double re = r < p->halo_cutoff ? r : p->halo_cutoff;
    double x = re / p->halo_a;
    return p->halo_GM * pow(x, p->halo_gamma) / (1.0 + pow(x, p->halo_gamma - 1.0));
}

static void mw_accel(const Potential *pot, Vec3 q, Vec3 *out) {
    const MilkyWayParams *p = (const MilkyWayParams *)pot->params;
    double R2 = q.x * q.x + q.y * q.y, R = sqrt(R2), r = vlen(q);
    Vec3 acc = vmk(0, 0, 0);
    double den = pow(r * r + p->bulge_b * p->bulge_b, 1.5);          /* Plummer bulge */
    acc = vplus(acc, vtimes(q, -p->bulge_GM / (den > 0 ? den : 1e-12)));
    double zeta = sqrt(q.z * q.z + p->disk_b * p->disk_b);            /* Miyamoto-Nagai disk */
    double az_ = p->disk_a + zeta;
    double D2 = R2 + az_ * az_, D = sqrt(D2), D3 = D2 * D;
    double aR = -p->disk_GM * R / D3;
    double az = -p->disk_GM * q.z * az_ / (zeta > 0 ? zeta : 1e-12) / D3;
    if (R > 1e-12) { acc.x += aR * q.x / R; acc.y += aR * q.y / R; }
    acc.z += az;
    double rs = r > 1e-12 ? r : 1e-12;                                /* truncated halo */
    acc = vplus(acc, vtimes(q, -halo_mass(p, rs) / (rs * rs * rs)));
    *out = acc;
}

static double mw_energy(const Potential *pot, Vec3 q) {                /* reference src/potential.c:103-135 */
    const MilkyWayParams *p = (const MilkyWayParams *)pot->params;
    double R2 = q.x * q.x + q.y * q.y, r = vlen(q);
    double e_b = -p->bulge_GM / sqrt(r * r + p->bulge_b * p->bulge_b);
    double zeta = sqrt(q.z * q.z + p->disk_b * p->disk_b), az_ = p->disk_a + zeta;
    double e_d = -p->disk_GM / sqrt(R2 + az_ * az_);
    double rs = r > 1e-12 ? r : 1e-12, mL = halo_mass(p, p->halo_cutoff), e_h;
    if (rs >= p->halo_cutoff) e_h = -mL / rs;
    else {
        double g1 = p->halo_gamma - 1.0, xL = p->halo_cutoff / p->halo_a, xr = rs / p->halo_a;
        double I = (1.0 / g1) * (log(1.0 + pow(xL, g1)) - log(1.0 + pow(xr, g1)));
        e_h = -(p->halo_GM / p->halo_a) * I - mL / p->halo_cutoff;
    }
    return e_b + e_d + e_h;
}

static Potential g_mw;
static Vec3 g_sun_x, g_sun_v;

static Vec3 accel(Vec3 q) { Vec3 a; g_mw.acceleration(&g_mw, q, &a); return a; }

/* ---- coordinates (reference src/coords.c:33-40, 77-131) ----------------------------------------------------- */
static Vec3 rotate(Vec3 v) {
    return vmk(ROT[0][0] * v.x + ROT[0][1] * v.y + ROT[0][2] * v.z,
               ROT[1][0] * v.x + ROT[1][1] * v.y + ROT[1][2] * v.z,
               ROT[2][0] * v.x + ROT[2][1] * v.y + ROT[2][2] * v.z);
}
static Vec3 helio_pos(Vec3 v, const SolarParams *s) {
    Vec3 g = rotate(v);
    return vmk(g.x - s->r0_kpc, g.y, g.z + s->z0_kpc);
}
static Vec3 helio_vel(Vec3 v, const SolarParams *s) {
    Vec3 g = rotate(v);
    Vec3 sun = vmk(s->u_pec_kms / KMS_PER_KPCMYR, (s->v_circ_kms + s->v_pec_kms) / KMS_PER_KPCMYR,
                   s->w_pec_kms / KMS_PER_KPCMYR);
    return vplus(g, sun);
}

static void to_galcen(Astrometry a, PhaseSpace *out) {
    const SolarParams *s = &solar_params_default;
    double ra = a.ra_deg * DEG_TO_RAD, dec = a.dec_deg * DEG_TO_RAD;
    double dk = 1.0 / a.parallax_mas, dpc = dk * 1000.0;
    double cd = cos(dec), sd = sin(dec), cr = cos(ra), sr = sin(ra);
    Vec3 er = vmk(cd * cr, cd * sr, sd);
    Vec3 ea = vmk(-sr, cr, 0.0);
    Vec3 ed = vmk(-sd * cr, -sd * sr, cd);
    out->pos = helio_pos(vtimes(er, dk), s);
    double va = AU_PER_YR_KMS * 1e-3 * a.pmra_masyr * dpc;
    double vd = AU_PER_YR_KMS * 1e-3 * a.pmdec_masyr * dpc;
    Vec3 v = vplus(vplus(vtimes(er, a.rv_kms), vtimes(ea, va)), vtimes(ed, vd));
    out->vel = helio_vel(vmk(v.x / KMS_PER_KPCMYR, v.y / KMS_PER_KPCMYR, v.z / KMS_PER_KPCMYR), s);
}

/* ---- random numbers (reference src/montecarlo.h:26-41, src/montecarlo.c:4-17) -------------------------------- */
static uint64_t sm64(McRng *g) {
    uint64_t z = (g->state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double unif(McRng *g) { return (double)(sm64(g) >> 11) * (1.0 / 9007199254740992.0); }
static double normal(McRng *g) {
    double u1 = unif(g);
    if (u1 <= 0.0) u1 = 1.0 / 18446744073709551616.0;
    double u2 = unif(g);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * PI_LIT * u2);
}
static double gz(McRng *g) { return g ? normal(g) : 0.0; }

/* ---- draws (reference src/phygas.c:12-82) --------------------------------------------------------------------- */
void ph_init(void) {
    g_mw.acceleration = mw_accel;
    g_mw.energy = mw_energy;
    g_mw.params = &milkyway_potential_default;
    Vec3 o = vmk(0, 0, 0);
    g_sun_x = helio_pos(o, &solar_params_default);
    g_sun_v = helio_vel(o, &solar_params_default);
}

const Potential *ph_potential(void) { return &g_mw; }

static double rv_prior_centre(Vec3 q) {
    double R = hypot(q.x, q.y);
    if (R <= 0) return 0.0;
    Vec3 a = accel(vmk(q.x, q.y, 0.0));
    double ar = -(a.x * q.x + a.y * q.y) / R;
    double vc = ar > 0 ? sqrt(R * ar) : 0.0;
    Vec3 v = vmk(vc * q.y / R, -vc * q.x / R, 0.0);
    Vec3 los = vminus(q, g_sun_x);
    double n = vlen(los);
    if (n <= 0) return 0.0;
    return vdot(vminus(v, g_sun_v), vtimes(los, 1.0 / n)) * KMS_PER_KPCMYR;
}

static void with_rv(Astrometry a, int has_rv, double rv, double e_rv, double prior, McRng *g, PhaseSpace *out) {
    if (has_rv) {
        a.rv_kms = rv + e_rv * gz(g);
    } else {
        PhaseSpace p0;
        a.rv_kms = 0.0;
        to_galcen(a, &p0);
        a.rv_kms = rv_prior_centre(p0.pos) + prior * gz(g);
    }
    to_galcen(a, out);
}

int ph_sample_target(const PhTarget *t, McRng *g, PhaseSpace *out) {
    Astrometry a;
    a.ra_deg = t->ra; a.dec_deg = t->dec;
    for (int attempt = 0; attempt < 50; attempt++) {
        double plx = t->plx > 0 ? t->plx + t->e_plx * gz(g)
                                : 1000.0 / (t->dist_pc * exp(t->e_lndist * gz(g)));
        if (!(plx > 0)) continue;
        a.parallax_mas = plx;
        a.pmra_masyr = t->pmra + t->e_pmra * gz(g);
        a.pmdec_masyr = t->pmdec + t->e_pmdec * gz(g);
        with_rv(a, t->has_rv, t->rv, t->e_rv, t->kind == 'P' ? PH_PULSAR_RV_PRIOR : PH_STAR_RV_PRIOR, g, out);
        return 0;
    }
    return -1;
}

int ph_sample_cluster(const PhCluster *c, McRng *g, PhaseSpace *out) {
    Astrometry a;
    a.ra_deg = c->ra; a.dec_deg = c->dec;
    for (int attempt = 0; attempt < 50; attempt++) {
        double d = c->dist_pc + c->e_dist_pc * gz(g);
        if (!(d > 0)) continue;
        a.parallax_mas = 1000.0 / d;
        a.pmra_masyr = c->pmra + c->e_pmra * gz(g);
        a.pmdec_masyr = c->pmdec + c->e_pmdec * gz(g);
        with_rv(a, c->has_rv, c->rv, c->e_rv, PH_CLUSTER_RV_PRIOR, g, out);
        return 0;
    }
    return -1;
}

/* ---- leapfrog, tracks, prefilter (reference src/phygas.c:84-168) --------------------------------------------- */
typedef struct { Vec3 x, v, a; } Orbit;

static void orbit_start(Orbit *o, PhaseSpace s) { o->x = s.pos; o->v = s.vel; o->a = accel(s.pos); }
static void kdk(Orbit *o, double dt) {
    double h = 0.5 * dt;
    o->v = vplus(o->v, vtimes(o->a, h));
    o->x = vplus(o->x, vtimes(o->v, dt));
    o->a = accel(o->x);
    o->v = vplus(o->v, vtimes(o->a, h));
}

static void coarse_track(PhaseSpace s, double tmax, PhTrack *out) {
    int n = (int)ceil(tmax / PH_PRE_STEP_MYR) + 1;
    double dt = -PH_PRE_STEP_MYR / 10;
    Orbit o;
    out->n = n;
    out->pos = malloc(sizeof(Vec3) * n);
    orbit_start(&o, s);
    out->pos[0] = o.x;
    for (int k = 1; k < n; k++) {
        for (int i = 0; i < 10; i++) kdk(&o, dt);
        out->pos[k] = o.x;
    }
}

static void clone_spread(PhaseSpace nom, const PhaseSpace *d, int n, PhTrack *out) {
    double sx = 0, sv = 0;
    for (int i = 0; i < n; i++) {
        Vec3 dx = vminus(d[i].pos, nom.pos), dv = vminus(d[i].vel, nom.vel);
        sx += vdot(dx, dx);
        sv += vdot(dv, dv);
    }
    out->sig_pos = n ? sqrt(sx / n) : 0;
    out->sig_vel = n ? sqrt(sv / n) : 0;
}

void ph_track_target(const PhTarget *t, double tmax, int n_spread, uint64_t seed, PhTrack *out) {
    PhaseSpace nom, d[64];
    McRng g;
    int k = 0;
    ph_sample_target(t, NULL, &nom);
    g.state = seed;
    if (n_spread > 64) n_spread = 64;
    for (int i = 0; i < n_spread; i++) if (ph_sample_target(t, &g, &d[k]) == 0) k++;
    coarse_track(nom, tmax, out);
    clone_spread(nom, d, k, out);
}

void ph_track_cluster(const PhCluster *c, int n_spread, uint64_t seed, PhTrack *out) {
    PhaseSpace nom, d[64];
    McRng g;
    int k = 0;
    ph_sample_cluster(c, NULL, &nom);
    g.state = seed;
    if (n_spread > 64) n_spread = 64;
    for (int i = 0; i < n_spread; i++) if (ph_sample_cluster(c, &g, &d[k]) == 0) k++;
    coarse_track(nom, c->tmax_myr, out);
    clone_spread(nom, d, k, out);
}

void ph_track_free(PhTrack *t) { free(t->pos); t->pos = NULL; t->n = 0; }

/* nearest point of the segment r0 -> r1 to the origin: distance, and where (s in [0,1]) */
static double seg_near(Vec3 r0, Vec3 r1, double *s_out) {
    Vec3 dr = vminus(r1, r0);
    double dd = vdot(dr, dr), s = 0;
    if (dd > 0) {
        s = -vdot(r0, dr) / dd;
        if (s < 0) s = 0; else if (s > 1) s = 1;
    }
    *s_out = s;
    return vlen(vplus(r0, vtimes(dr, s)));
}

int ph_prefilter(const PhTrack *tt, const PhTrack *ct, const PhCluster *c) {
    int n = tt->n < ct->n ? tt->n : ct->n;
    double sx = hypot(tt->sig_pos, ct->sig_pos), sv = hypot(tt->sig_vel, ct->sig_vel);
    double reach = (3.0 * c->rtot_pc + 10.0) / 1000.0;
    for (int k = 0; k + 1 < n; k++) {
        double s, d = seg_near(vminus(tt->pos[k], ct->pos[k]), vminus(tt->pos[k + 1], ct->pos[k + 1]), &s);
        double tk = (k + s) * PH_PRE_STEP_MYR;
        if (d < reach + 3.0 * (sx + sv * tk)) return 1;
    }
    return 0;
}

/* ---- pair Monte Carlo (reference src/phygas.c:170-249) ------------------------------------------------------- */
static int by_value(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

static double interp_quantile(const double *v, int n, double q) {
    double pos = q * (n - 1);
    int i = (int)pos;
    if (i >= n - 1) return v[n - 1];
    return v[i] + (pos - i) * (v[i + 1] - v[i]);
}

int ph_pair_draw(const PhTarget *t, const PhCluster *c, int n_clones, double dt_myr, uint64_t seed, double *ps,
                 int *steps_out, double *dt_out) {
    McRng g;
    int steps = (int)ceil(c->tmax_myr / dt_myr), m = 0;
    g.state = seed;
    *steps_out = steps;
    *dt_out = -c->tmax_myr / steps;
    for (int k = 0; k < n_clones; k++) {
        PhaseSpace a, b;
        if (ph_sample_target(t, &g, &a) || ph_sample_cluster(c, &g, &b)) continue;
        double *o = ps + (size_t)m * 12;
        o[0] = a.pos.x; o[1] = a.pos.y; o[2] = a.pos.z; o[3] = a.vel.x; o[4] = a.vel.y; o[5] = a.vel.z;
        o[6] = b.pos.x; o[7] = b.pos.y; o[8] = b.pos.z; o[9] = b.vel.x; o[10] = b.vel.y; o[11] = b.vel.z;
        m++;
    }
    return m;
}

void ph_pair_clone(const double *ps, int steps, double dt, double *best_out, double *tbest_out, double *vbest_out) {
    PhaseSpace pa, pb;
    Orbit a, b;
    pa.pos = vmk(ps[0], ps[1], ps[2]); pa.vel = vmk(ps[3], ps[4], ps[5]);
    pb.pos = vmk(ps[6], ps[7], ps[8]); pb.vel = vmk(ps[9], ps[10], ps[11]);
    orbit_start(&a, pa);
    orbit_start(&b, pb);
    Vec3 r0 = vminus(a.x, b.x);
    double best = vlen(r0), tbest = 0, vbest = vlen(vminus(a.v, b.v));
    for (int i = 1; i <= steps; i++) {
        kdk(&a, dt);
        kdk(&b, dt);
        Vec3 r1 = vminus(a.x, b.x);
        double s, d = seg_near(r0, r1, &s);
        if (d < best) {
            best = d;
            tbest = (i - 1 + s) * -dt;
            vbest = vlen(vminus(a.v, b.v));
        }
        r0 = r1;
    }
    *best_out = best; *tbest_out = tbest; *vbest_out = vbest;
}

void ph_pair_reduce(const PhCluster *c, int m, const double *best, const double *tbest, const double *vbest,
                    PhResult *res) {
    int cap = m > 0 ? m : 1, in50 = 0, intot = 0;
    double *d = malloc(sizeof(double) * cap * 3), *t = d + cap, *v = d + 2 * cap;
    for (int k = 0; k < m; k++) {
        d[k] = best[k] * 1000.0;
        t[k] = tbest[k];
        v[k] = vbest[k] * KMS_PER_KPCMYR;
        if (d[k] < c->r50_pc) in50++;
        if (d[k] < c->rtot_pc) intot++;
    }
    memset(res, 0, sizeof(*res));
    res->n = m;
    if (m > 0) {
        res->f_r50 = (double)in50 / m;
        res->f_rtot = (double)intot / m;
        qsort(d, m, sizeof(double), by_value);
        qsort(t, m, sizeof(double), by_value);
        qsort(v, m, sizeof(double), by_value);
        res->d05 = interp_quantile(d, m, 0.05); res->d50 = interp_quantile(d, m, 0.5); res->d95 = interp_quantile(d, m, 0.95);
        res->t05 = interp_quantile(t, m, 0.05); res->t50 = interp_quantile(t, m, 0.5); res->t95 = interp_quantile(t, m, 0.95);
        res->v05 = interp_quantile(v, m, 0.05); res->v50 = interp_quantile(v, m, 0.5); res->v95 = interp_quantile(v, m, 0.95);
    }
    free(d);
}

void ph_pair(const PhTarget *t, const PhCluster *c, int n_clones, double dt_myr, uint64_t seed, PhResult *res) {
    int cap = n_clones > 0 ? n_clones : 1, steps;
    double *ps = malloc(sizeof(double) * 12 * cap), *r = malloc(sizeof(double) * 3 * cap), dt;
    int m = ph_pair_draw(t, c, n_clones, dt_myr, seed, ps, &steps, &dt);
    for (int k = 0; k < m; k++) ph_pair_clone(ps + (size_t)k * 12, steps, dt, &r[k], &r[m + k], &r[2 * m + k]);
    ph_pair_reduce(c, m, r, r + m, r + 2 * m, res);
    free(ps);
    free(r);
}

/* ---- linear screen (reference src/phygas.c:251-450) ---------------------------------------------------------- */
static void draw_cov(PhaseSpace nom, const PhaseSpace *d, int nd, double sig[6][6]) {
    memset(sig, 0, sizeof(double[6][6]));
    for (int i = 0; i < nd; i++) {
        double e[6] = {d[i].pos.x - nom.pos.x, d[i].pos.y - nom.pos.y, d[i].pos.z - nom.pos.z,
                       d[i].vel.x - nom.vel.x, d[i].vel.y - nom.vel.y, d[i].vel.z - nom.vel.z};
        for (int a = 0; a < 6; a++) for (int b = 0; b < 6; b++) sig[a][b] += e[a] * e[b];
    }
    for (int a = 0; a < 6; a++) for (int b = 0; b < 6; b++) sig[a][b] /= nd > 0 ? nd : 1;
}

/* nominal orbit + one neighbour per phase-space axis; position covariance A Sigma0 A^T at every point */
static void stm_track(PhaseSpace nom, double sig[6][6], double tmax, PhLin *out) {
    Orbit o[7];
    orbit_start(&o[0], nom);
    for (int j = 0; j < 6; j++) {
        PhaseSpace p = nom;
        double e = j < 3 ? PH_LIN_EPS_POS : PH_LIN_EPS_VEL;
        switch (j) {
        case 0: p.pos.x += e; break;
        case 1: p.pos.y += e; break;
        case 2: p.pos.z += e; break;
        case 3: p.vel.x += e; break;
        case 4: p.vel.y += e; break;
        default: p.vel.z += e; break;
        }
        orbit_start(&o[j + 1], p);
    }
    int n = (int)ceil(tmax / PH_PRE_STEP_MYR) + 1;
    double dt = -PH_PRE_STEP_MYR / PH_LIN_SUB;
    out->n = n;
    out->pos = malloc(sizeof(Vec3) * n);
    out->vel = malloc(sizeof(Vec3) * n);
    out->S = malloc(sizeof(double[6]) * n);
    for (int k = 0; k < n; k++) {
        if (k > 0)
            for (int i = 0; i < PH_LIN_SUB; i++)
                for (int j = 0; j < 7; j++) kdk(&o[j], dt);
        out->pos[k] = o[0].x;
        out->vel[k] = o[0].v;
        double A[3][6], AS[3][6] = {{0}}, S[3][3] = {{0}};
        for (int j = 0; j < 6; j++) {
            double e = j < 3 ? PH_LIN_EPS_POS : PH_LIN_EPS_VEL;
            Vec3 d = vminus(o[j + 1].x, o[0].x);
            A[0][j] = d.x / e; A[1][j] = d.y / e; A[2][j] = d.z / e;
        }
        for (int r = 0; r < 3; r++)
            for (int b = 0; b < 6; b++)
                for (int a = 0; a < 6; a++) AS[r][b] += A[r][a] * sig[a][b];
        for (int r = 0; r < 3; r++)
            for (int s = 0; s < 3; s++)
                for (int b = 0; b < 6; b++) S[r][s] += AS[r][b] * A[s][b];
        out->S[k][0] = S[0][0]; out->S[k][1] = S[0][1]; out->S[k][2] = S[0][2];
        out->S[k][3] = S[1][1]; out->S[k][4] = S[1][2]; out->S[k][5] = S[2][2];
    }
}

void ph_lin_target_init(const PhTarget *t, int n_samp, uint64_t seed, double ps0[6], double sig[6][6]) {
    PhaseSpace nom, *d = malloc(sizeof(PhaseSpace) * (n_samp > 0 ? n_samp : 1));
    McRng g;
    int k = 0;
    ph_sample_target(t, NULL, &nom);
    g.state = seed;
    for (int i = 0; i < n_samp; i++) if (ph_sample_target(t, &g, &d[k]) == 0) k++;
    draw_cov(nom, d, k, sig);
    free(d);
    ps0[0] = nom.pos.x; ps0[1] = nom.pos.y; ps0[2] = nom.pos.z;
    ps0[3] = nom.vel.x; ps0[4] = nom.vel.y; ps0[5] = nom.vel.z;
}

void ph_lin_target(const PhTarget *t, double tmax, int n_samp, uint64_t seed, PhLin *out) {
    double ps0[6], sig[6][6];
    PhaseSpace nom;
    ph_lin_target_init(t, n_samp, seed, ps0, sig);
    nom.pos = vmk(ps0[0], ps0[1], ps0[2]);
    nom.vel = vmk(ps0[3], ps0[4], ps0[5]);
    stm_track(nom, sig, tmax, out);
}

void ph_lin_cluster(const PhCluster *c, int n_samp, uint64_t seed, PhLin *out) {
    PhaseSpace nom, *d = malloc(sizeof(PhaseSpace) * (n_samp > 0 ? n_samp : 1));
    McRng g;
    double sig[6][6];
    int k = 0;
    ph_sample_cluster(c, NULL, &nom);
    g.state = seed;
    for (int i = 0; i < n_samp; i++) if (ph_sample_cluster(c, &g, &d[k]) == 0) k++;
    draw_cov(nom, d, k, sig);
    free(d);
    stm_track(nom, sig, c->tmax_myr, out);
}

void ph_lin_free(PhLin *l) {
    free(l->pos); free(l->vel); free(l->S);
    l->pos = l->vel = NULL; l->S = NULL; l->n = 0;
}

/* m^T M^-1 m for symmetric M (xx xy xz yy yz zz) by the adjugate; -1 when det <= 0 */
static double inv_form(const double M[6], Vec3 m) {
    double a = M[0], b = M[1], c = M[2], d = M[3], e = M[4], f = M[5];
    double c00 = d * f - e * e, c01 = c * e - b * f, c02 = b * e - c * d;
    double det = a * c00 + b * c01 + c * c02;
    if (!(det > 0)) return -1;
    double c11 = a * f - c * c, c12 = b * c - a * e, c22 = a * d - b * b;
    return (m.x * (c00 * m.x + c01 * m.y + c02 * m.z) + m.y * (c01 * m.x + c11 * m.y + c12 * m.z)
            + m.z * (c02 * m.x + c12 * m.y + c22 * m.z)) / det;
}

double ph_screen_r = 2.0;

double ph_screen_chi2_cut(const PhLin *tl, const PhLin *cl, const PhCluster *c, double cut, int *kb_out,
                          double *sb_out) {
    int n = tl->n < cl->n ? tl->n : cl->n, kb = 0;
    double R = (ph_screen_r > 0 ? ph_screen_r * c->r50_pc : c->rtot_pc) / 1000.0, R2 = R * R;
    double best = INFINITY, sb = 0;
    for (int k = 0; k < n; k++) {
        double M[6];
        for (int i = 0; i < 6; i++) M[i] = tl->S[k][i] + cl->S[k][i];
        M[0] += R2; M[3] += R2; M[5] += R2;
        Vec3 m0 = vminus(tl->pos[k], cl->pos[k]), m1 = m0;
        if (k + 1 < n) m1 = vminus(tl->pos[k + 1], cl->pos[k + 1]);
        double thr = 2.0 * cut * (M[0] + M[3] + M[5]);
        if (thr < INFINITY) {       /* early reject: chi2 at this point >= dist^2 / trace(M) (reference :360-394) */
            Vec3 dr = vminus(m1, m0);
            double a = vdot(m0, dr), dd = vdot(dr, dr);
            int far;
            if (a >= 0) far = vdot(m0, m0) > thr;
            else if (-a >= dd) far = vdot(m1, m1) > thr;
            else far = vdot(m0, m0) * dd - a * a > thr * dd;
            if (far) continue;
        }
        double q = inv_form(M, m0), s = 0;
        if (k + 1 < n) {
            seg_near(m0, m1, &s);
            double qs = inv_form(M, vplus(m0, vtimes(vminus(m1, m0), s)));
            if (qs >= 0 && qs < q) q = qs; else s = 0;
        }
        if (q >= 0 && q < best) { best = q; kb = k; sb = s; }
    }
    *kb_out = kb;
    *sb_out = sb;
    return best;
}

double ph_screen_chi2(const PhLin *tl, const PhLin *cl, const PhCluster *c, int *kb, double *sb) {
    return ph_screen_chi2_cut(tl, cl, c, INFINITY, kb, sb);
}

void ph_screen_finish(const PhLin *tl, const PhLin *cl, const PhCluster *c, uint64_t seed, double chi2, int kb,
                      double sb, PhScreen *res) {
    int n = tl->n < cl->n ? tl->n : cl->n, k1 = kb + 1 < n ? kb + 1 : kb;
    memset(res, 0, sizeof(*res));
    res->chi2 = chi2;
    res->t = (kb + sb) * PH_PRE_STEP_MYR;
    Vec3 a = vminus(tl->pos[kb], cl->pos[kb]);
    Vec3 m = vplus(a, vtimes(vminus(vminus(tl->pos[k1], cl->pos[k1]), a), sb));
    res->d_nom_pc = vlen(m) * 1000.0;
    res->vrel = vlen(vminus(tl->vel[kb], cl->vel[kb])) * KMS_PER_KPCMYR;
    double C[6];
    for (int i = 0; i < 6; i++) C[i] = tl->S[kb][i] + cl->S[kb][i];
    res->sig_pc = sqrt((C[0] + C[3] + C[5]) / 3.0) * 1000.0;
    double l00 = sqrt(fmax(C[0], 0)), l10 = l00 > 0 ? C[1] / l00 : 0, l20 = l00 > 0 ? C[2] / l00 : 0;
    double l11 = sqrt(fmax(C[3] - l10 * l10, 0)), l21 = l11 > 0 ? (C[4] - l20 * l10) / l11 : 0;
    double l22 = sqrt(fmax(C[5] - l20 * l20 - l21 * l21, 0));
    double r50 = c->r50_pc / 1000.0, rt = c->rtot_pc / 1000.0;
    McRng g;
    int in50 = 0, intot = 0;
    g.state = seed;
    for (int i = 0; i < 512; i++) {
        double z0 = normal(&g), z1 = normal(&g), z2 = normal(&g);
        double r = vlen(vmk(m.x + l00 * z0, m.y + l10 * z0 + l11 * z1, m.z + l20 * z0 + l21 * z1 + l22 * z2));
        if (r < r50) in50++;
        if (r < rt) intot++;
    }
    res->p_r50 = (double)in50 / 512;
    res->p_rtot = (double)intot / 512;
}

void ph_screen(const PhLin *tl, const PhLin *cl, const PhCluster *c, uint64_t seed, PhScreen *res) {
    int kb;
    double sb, best = ph_screen_chi2(tl, cl, c, &kb, &sb);
    ph_screen_finish(tl, cl, c, seed, best, kb, sb, res);
}

uint64_t ph_seed(const char *a, const char *b) {
    uint64_t h = 1469598103934665603ULL;              /* FNV-1a offset basis over "a|b" */
    for (const unsigned char *p = (const unsigned char *)a; *p; p++) h = (h ^ *p) * 1099511628211ULL;
    h = (h ^ (unsigned char)'|') * 1099511628211ULL;
    for (const unsigned char *p = (const unsigned char *)b; *p; p++) h = (h ^ *p) * 1099511628211ULL;
    return h;
}

/* ---- readers (reference src/phygas.c:460-506): whitespace text, a line that does not parse is skipped ------- */
static double field_value(const char *s) { return strcmp(s, "nan") == 0 ? NAN : atof(s); }

int ph_read_clusters(const char *path, PhCluster **out) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    int cap = 1024, n = 0, idx;
    PhCluster *v = malloc(sizeof(PhCluster) * cap);
    char line[1024], srv[32], serv[32], kind[4];
    while (fgets(line, sizeof line, f)) {
        if (n == cap) { cap *= 2; v = realloc(v, sizeof(PhCluster) * cap); }
        PhCluster *c = &v[n];
        if (sscanf(line, "%d %39s %3s %lf %lf %lf %lf %lf %lf %lf %lf %31s %31s %lf %lf %lf %lf %lf %lf", &idx,
                   c->name, kind, &c->ra, &c->dec, &c->dist_pc, &c->e_dist_pc, &c->pmra, &c->e_pmra, &c->pmdec,
                   &c->e_pmdec, srv, serv, &c->r50_pc, &c->rtot_pc, &c->age16, &c->age50, &c->age84,
                   &c->tmax_myr) != 19)
            continue;
        c->kind = kind[0];
        c->rv = field_value(srv);
        c->e_rv = field_value(serv);
        c->has_rv = !isnan(c->rv) && !isnan(c->e_rv);
        n++;
    }
    fclose(f);
    *out = v;
    return n;
}

int ph_read_targets(const char *path, PhTarget **out) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    int cap = 1024, n = 0;
    PhTarget *v = malloc(sizeof(PhTarget) * cap);
    char line[1024], srv[32], serv[32], kind[4];
    while (fgets(line, sizeof line, f)) {
        if (n == cap) { cap *= 2; v = realloc(v, sizeof(PhTarget) * cap); }
        PhTarget *t = &v[n];
        if (sscanf(line, "%39s %3s %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %31s %31s", t->id, kind, &t->ra, &t->dec,
                   &t->plx, &t->e_plx, &t->dist_pc, &t->e_lndist, &t->pmra, &t->e_pmra, &t->pmdec, &t->e_pmdec, srv,
                   serv) != 14)
            continue;
        t->kind = kind[0];
        t->rv = field_value(srv);
        t->e_rv = field_value(serv);
        t->has_rv = !isnan(t->rv) && !isnan(t->e_rv);
        n++;
    }
    fclose(f);
    *out = v;
    return n;
}
