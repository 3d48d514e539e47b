/* ph_host.c -- host half of the Phygas C API in libphygas_gb300.
 *
 * Everything that sets the numbers' inputs stays on the host, as in the reference's GPU application
 * (src/main_phygas_boinc.cpp:29-34): the draws from measurement errors with their radial-velocity priors, the
 * 6-D covariance of the draws, the clone start states of ph_pair, the seeds and the file readers.  The draws must
 * equal the reference's bit for bit ("identical host-generated clone draws"), so this file evaluates every
 * expression in the reference's order and is built with -ffp-contract=off:
 *   force law       src/potential.c:53-101     (used here for the RV prior and the coarse tracks)
 *   astrometry      src/coords.c:77-131
 *   splitmix64/BM   src/montecarlo.h:26-41, src/montecarlo.c:4-17
 *   draws           src/phygas.c:21-82
 *   tracks/prefilter src/phygas.c:98-168
 *   ph_pair_draw    src/phygas.c:182-198;  covariance src/phygas.c:256-284;  ph_seed :452-458;  readers :460-506
 * The orbit integrations, the scan, the probabilities and the clone Monte Carlo are in the CUDA part
 * (the .cu files under csrc/cuda) behind the batched C-ABI of phygas_gb300.h.
 */
#include "ph_host.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define KMS_KPCMYR 977.7922216807892
#define GRAV (4.30091e-6 / (KMS_KPCMYR * KMS_KPCMYR))
#define MGAL_MSUN 2.325e7
#define PI_D 3.14159265358979323846
#define RAD (PI_D / 180.0)
#define AUYR (1.495978707e8 / 3.15576e7)

const MilkyWayParams milkyway_potential_default = {
    GRAV * (606.0 * MGAL_MSUN), 0.3873, GRAV * (3690.0 * MGAL_MSUN), 5.3178, 0.2500,
    GRAV * (4615.0 * MGAL_MSUN), 12.0, 100.0, 2.02,
};
const SolarParams solar_params_default = {8.122, 0.0208, 229.0, 11.1, 12.24, 7.25};

static const double ICRS_TO_GAL[3][3] = {   /* Hipparcos (ESA 1997, vol. 1 sec. 1.5.3) */
    {-0.0548755604162154, -0.8734370902348850, -0.4838350155487132},
    {0.4941094278755837, -0.4448296299600112, 0.7469822444972189},
    {-0.8676661490190047, -0.1980763734312015, 0.4559837761750669},
};

double ph_screen_r = 2.0;

typedef struct { double x, y, z; } V3;
static inline V3 v3(double x, double y, double z) { V3 v = {x, y, z}; return v; }
static inline V3 add3(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 sub3(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 mul3(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline double dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double len3(V3 a) { return sqrt(dot3(a, a)); }
static inline V3 fromv(Vec3 a) { return v3(a.x, a.y, a.z); }
static inline Vec3 tov(V3 a) { Vec3 r; r.x = a.x; r.y = a.y; r.z = a.z; return r; }

/* ---- force law on the host (the GPU has its own, csrc/cuda/force.cuh) -------------------------------------- */
static double enclosed(const MilkyWayParams *p, double r) {
    double r_in = r < p->halo_cutoff ? r : p->halo_cutoff;
    double x = r_in / p->halo_a;
    return p->halo_GM * pow(x, p->halo_gamma) / (1.0 + pow(x, p->halo_gamma - 1.0));
}

static V3 host_accel(V3 q) {
    const MilkyWayParams *p = &milkyway_potential_default;
    double R2 = q.x * q.x + q.y * q.y, R = sqrt(R2), r = len3(q);
    V3 a = v3(0, 0, 0);
    double pl = pow(r * r + p->bulge_b * p->bulge_b, 1.5);
    a = add3(a, mul3(q, -p->bulge_GM / (pl > 0 ? pl : 1e-12)));
    double zeta = sqrt(q.z * q.z + p->disk_b * p->disk_b), s = p->disk_a + zeta;
    double D2 = R2 + s * s, D = sqrt(D2), D3 = D2 * D;
    double fR = -p->disk_GM * R / D3;
    double fz = -p->disk_GM * q.z * s / (zeta > 0 ? zeta : 1e-12) / D3;
    if (R > 1e-12) { a.x += fR * q.x / R; a.y += fR * q.y / R; }
    a.z += fz;
    double rr = r > 1e-12 ? r : 1e-12;
    return add3(a, mul3(q, -enclosed(p, rr) / (rr * rr * rr)));
}

static void pot_accel(const Potential *pot, Vec3 pos, Vec3 *out) { (void)pot; *out = tov(host_accel(fromv(pos))); }
static double pot_energy(const Potential *pot, Vec3 pos) {
    (void)pot;
    const MilkyWayParams *p = &milkyway_potential_default;
    V3 q = fromv(pos);
    double R2 = q.x * q.x + q.y * q.y, r = len3(q);
    double eb = -p->bulge_GM / sqrt(r * r + p->bulge_b * p->bulge_b);
    double zeta = sqrt(q.z * q.z + p->disk_b * p->disk_b), s = p->disk_a + zeta;
    double ed = -p->disk_GM / sqrt(R2 + s * s);
    double rr = r > 1e-12 ? r : 1e-12, mcut = enclosed(p, p->halo_cutoff), eh;
    if (rr >= p->halo_cutoff) eh = -mcut / rr;
    else {
        double g1 = p->halo_gamma - 1.0, xc = p->halo_cutoff / p->halo_a, xr = rr / p->halo_a;
        eh = -(p->halo_GM / p->halo_a) * ((1.0 / g1) * (log(1.0 + pow(xc, g1)) - log(1.0 + pow(xr, g1))))
             - mcut / p->halo_cutoff;
    }
    return eb + ed + eh;
}

static Potential g_pot = {pot_accel, pot_energy, &milkyway_potential_default};
static V3 g_sun_pos, g_sun_vel;
static int g_ready;

/* ---- astrometry -> Galactocentric phase space --------------------------------------------------------------- */
static V3 icrs_to_gal(V3 v) {
    const double (*m)[3] = ICRS_TO_GAL;
    return v3(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
              m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
}
static V3 sun_offset_pos(V3 g, const SolarParams *s) { return v3(g.x - s->r0_kpc, g.y, g.z + s->z0_kpc); }
static V3 sun_offset_vel(V3 g, const SolarParams *s) {
    return add3(g, v3(s->u_pec_kms / KMS_KPCMYR, (s->v_circ_kms + s->v_pec_kms) / KMS_KPCMYR, s->w_pec_kms / KMS_KPCMYR));
}

static void galcen(const Astrometry *a, V3 *pos, V3 *vel) {
    const SolarParams *s = &solar_params_default;
    double ra = a->ra_deg * RAD, dec = a->dec_deg * RAD;
    double d_kpc = 1.0 / a->parallax_mas, d_pc = d_kpc * 1000.0;
    V3 e_r = v3(cos(dec) * cos(ra), cos(dec) * sin(ra), sin(dec));
    V3 e_a = v3(-sin(ra), cos(ra), 0.0);
    V3 e_d = v3(-sin(dec) * cos(ra), -sin(dec) * sin(ra), cos(dec));
    *pos = sun_offset_pos(icrs_to_gal(mul3(e_r, d_kpc)), s);
    double va = AUYR * 1e-3 * a->pmra_masyr * d_pc, vd = AUYR * 1e-3 * a->pmdec_masyr * d_pc;
    V3 v = add3(add3(mul3(e_r, a->rv_kms), mul3(e_a, va)), mul3(e_d, vd));
    *vel = sun_offset_vel(icrs_to_gal(v3(v.x / KMS_KPCMYR, v.y / KMS_KPCMYR, v.z / KMS_KPCMYR)), s);
}

/* ---- random numbers ---------------------------------------------------------------------------------------- */
static inline uint64_t mix_next(McRng *g) {
    uint64_t z = (g->state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline double uniform53(McRng *g) { return (double)(mix_next(g) >> 11) * (1.0 / 9007199254740992.0); }
static double box_muller(McRng *g) {
    double u1 = uniform53(g);
    if (u1 <= 0.0) u1 = 1.0 / 18446744073709551616.0;
    double u2 = uniform53(g);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * PI_D * u2);
}
static inline double g_or_zero(McRng *g) { return g ? box_muller(g) : 0.0; }

/* ---- draws ----------------------------------------------------------------------------------------------------- */
void ph_init(void) {
    V3 zero = v3(0, 0, 0);
    g_sun_pos = sun_offset_pos(icrs_to_gal(zero), &solar_params_default);
    g_sun_vel = sun_offset_vel(icrs_to_gal(zero), &solar_params_default);
    g_ready = 1;
}
const Potential *ph_potential(void) { return &g_pot; }
static pthread_once_t g_once = PTHREAD_ONCE_INIT;
static void init_once(void) { ph_init(); }
static void ensure_init(void) { if (!g_ready) pthread_once(&g_once, init_once); }

static double rv_rotation(V3 q) {           /* RV of a circular orbit at q, seen from the Sun (reference :23-35) */
    double R = hypot(q.x, q.y);
    if (R <= 0) return 0.0;
    V3 a = host_accel(v3(q.x, q.y, 0.0));
    double ar = -(a.x * q.x + a.y * q.y) / R;
    double vc = ar > 0 ? sqrt(R * ar) : 0.0;
    V3 v = v3(vc * q.y / R, -vc * q.x / R, 0.0);
    V3 los = sub3(q, g_sun_pos);
    double n = len3(los);
    if (n <= 0) return 0.0;
    return dot3(sub3(v, g_sun_vel), mul3(los, 1.0 / n)) * KMS_KPCMYR;
}

static void close_draw(Astrometry a, int has_rv, double rv, double e_rv, double prior, McRng *g, PhaseSpace *out) {
    V3 p, v;
    if (has_rv) {
        a.rv_kms = rv + e_rv * g_or_zero(g);
    } else {
        a.rv_kms = 0.0;
        galcen(&a, &p, &v);
        a.rv_kms = rv_rotation(p) + prior * g_or_zero(g);
    }
    galcen(&a, &p, &v);
    out->pos = tov(p);
    out->vel = tov(v);
}

int ph_sample_target(const PhTarget *t, McRng *g, PhaseSpace *out) {
    Astrometry a;
    ensure_init();
    a.ra_deg = t->ra; a.dec_deg = t->dec;
    for (int tries = 0; tries < 50; tries++) {
        double plx = t->plx > 0 ? t->plx + t->e_plx * g_or_zero(g)
                                : 1000.0 / (t->dist_pc * exp(t->e_lndist * g_or_zero(g)));
        if (!(plx > 0)) continue;
        a.parallax_mas = plx;
        a.pmra_masyr = t->pmra + t->e_pmra * g_or_zero(g);
        a.pmdec_masyr = t->pmdec + t->e_pmdec * g_or_zero(g);
        close_draw(a, t->has_rv, t->rv, t->e_rv, t->kind == 'P' ? PH_PULSAR_RV_PRIOR : PH_STAR_RV_PRIOR, g, out);
        return 0;
    }
    return -1;
}

int ph_sample_cluster(const PhCluster *c, McRng *g, PhaseSpace *out) {
    Astrometry a;
    ensure_init();
    a.ra_deg = c->ra; a.dec_deg = c->dec;
    for (int tries = 0; tries < 50; tries++) {
        double d = c->dist_pc + c->e_dist_pc * g_or_zero(g);
        if (!(d > 0)) continue;
        a.parallax_mas = 1000.0 / d;
        a.pmra_masyr = c->pmra + c->e_pmra * g_or_zero(g);
        a.pmdec_masyr = c->pmdec + c->e_pmdec * g_or_zero(g);
        close_draw(a, c->has_rv, c->rv, c->e_rv, PH_CLUSTER_RV_PRIOR, g, out);
        return 0;
    }
    return -1;
}

/* nominal state + 6-D covariance of n_samp draws (reference lin_cov, src/phygas.c:256-265) */
static void nominal_and_cov(const PhaseSpace *nom, const PhaseSpace *d, int k, double ps0[6], double sig[36]) {
    memset(sig, 0, sizeof(double) * 36);
    for (int i = 0; i < k; i++) {
        double e[6] = {d[i].pos.x - nom->pos.x, d[i].pos.y - nom->pos.y, d[i].pos.z - nom->pos.z,
                       d[i].vel.x - nom->vel.x, d[i].vel.y - nom->vel.y, d[i].vel.z - nom->vel.z};
        for (int a = 0; a < 6; a++) for (int b = 0; b < 6; b++) sig[6 * a + b] += e[a] * e[b];
    }
    for (int a = 0; a < 36; a++) sig[a] /= k > 0 ? k : 1;
    ps0[0] = nom->pos.x; ps0[1] = nom->pos.y; ps0[2] = nom->pos.z;
    ps0[3] = nom->vel.x; ps0[4] = nom->vel.y; ps0[5] = nom->vel.z;
}

void pgh_target_init(const PhTarget *t, int n_samp, uint64_t seed, double ps0[6], double sig[36]) {
    PhaseSpace nom, stack[128], *d = n_samp <= 128 ? stack : malloc(sizeof(PhaseSpace) * n_samp);
    McRng g;
    int k = 0;
    ph_sample_target(t, NULL, &nom);
    g.state = seed;
    for (int i = 0; i < n_samp; i++) if (ph_sample_target(t, &g, &d[k]) == 0) k++;
    nominal_and_cov(&nom, d, k, ps0, sig);
    if (d != stack) free(d);
}

void pgh_cluster_init(const PhCluster *c, int n_samp, uint64_t seed, double ps0[6], double sig[36]) {
    PhaseSpace nom, stack[128], *d = n_samp <= 128 ? stack : malloc(sizeof(PhaseSpace) * n_samp);
    McRng g;
    int k = 0;
    ph_sample_cluster(c, NULL, &nom);
    g.state = seed;
    for (int i = 0; i < n_samp; i++) if (ph_sample_cluster(c, &g, &d[k]) == 0) k++;
    nominal_and_cov(&nom, d, k, ps0, sig);
    if (d != stack) free(d);
}

void ph_lin_target_init(const PhTarget *t, int n_samp, uint64_t seed, double ps0[6], double sig[6][6]) {
    pgh_target_init(t, n_samp, seed, ps0, &sig[0][0]);
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

/* ---- coarse tracks and the prefilter (host; they decide which pairs a pulsar job runs) ----------------------- */
typedef struct { V3 x, v, a; } Body;
static void body_from(Body *b, PhaseSpace s) { b->x = fromv(s.pos); b->v = fromv(s.vel); b->a = host_accel(b->x); }
static void body_kdk(Body *b, double dt) {
    double h = 0.5 * dt;
    b->v = add3(b->v, mul3(b->a, h));
    b->x = add3(b->x, mul3(b->v, dt));
    b->a = host_accel(b->x);
    b->v = add3(b->v, mul3(b->a, h));
}

static void coarse(PhaseSpace s, double tmax, PhTrack *out) {
    int n = (int)ceil(tmax / PH_PRE_STEP_MYR) + 1;
    double dt = -PH_PRE_STEP_MYR / 10;
    Body b;
    out->n = n;
    out->pos = malloc(sizeof(Vec3) * n);
    body_from(&b, s);
    out->pos[0] = tov(b.x);
    for (int k = 1; k < n; k++) {
        for (int i = 0; i < 10; i++) body_kdk(&b, dt);
        out->pos[k] = tov(b.x);
    }
}

static void spread_of(PhaseSpace nom, const PhaseSpace *d, int n, PhTrack *out) {
    double sp = 0, sv = 0;
    for (int i = 0; i < n; i++) {
        V3 dp = sub3(fromv(d[i].pos), fromv(nom.pos)), dv = sub3(fromv(d[i].vel), fromv(nom.vel));
        sp += dot3(dp, dp);
        sv += dot3(dv, dv);
    }
    out->sig_pos = n ? sqrt(sp / n) : 0;
    out->sig_vel = n ? sqrt(sv / n) : 0;
}

/* the nominal point and the draws of a track's spread (at most 64); returns how many draws succeeded */
static int track_draws_target(const PhTarget *t, int n_spread, uint64_t seed, PhaseSpace *nom, PhaseSpace d[64]) {
    McRng g;
    int k = 0;
    ph_sample_target(t, NULL, nom);
    g.state = seed;
    if (n_spread > 64) n_spread = 64;
    for (int i = 0; i < n_spread; i++) if (ph_sample_target(t, &g, &d[k]) == 0) k++;
    return k;
}

static int track_draws_cluster(const PhCluster *c, int n_spread, uint64_t seed, PhaseSpace *nom, PhaseSpace d[64]) {
    McRng g;
    int k = 0;
    ph_sample_cluster(c, NULL, nom);
    g.state = seed;
    if (n_spread > 64) n_spread = 64;
    for (int i = 0; i < n_spread; i++) if (ph_sample_cluster(c, &g, &d[k]) == 0) k++;
    return k;
}

void ph_track_target(const PhTarget *t, double tmax, int n_spread, uint64_t seed, PhTrack *out) {
    PhaseSpace nom, d[64];
    const int k = track_draws_target(t, n_spread, seed, &nom, d);
    coarse(nom, tmax, out);
    spread_of(nom, d, k, out);
}

void ph_track_cluster(const PhCluster *c, int n_spread, uint64_t seed, PhTrack *out) {
    PhaseSpace nom, d[64];
    const int k = track_draws_cluster(c, n_spread, seed, &nom, d);
    coarse(nom, c->tmax_myr, out);
    spread_of(nom, d, k, out);
}

typedef struct {
    const PhTarget *t;
    const PhCluster *c;
    double *ps, *sig;
} StartArg;

static void starts_range(void *p, int i0, int i1) {
    StartArg *A = p;
    for (int i = i0; i < i1; i++) {
        PhaseSpace nom, d[64];
        PhTrack s;
        const int k = A->t ? track_draws_target(&A->t[i], 32, ph_seed("track", A->t[i].id), &nom, d)
                           : track_draws_cluster(&A->c[i], 32, ph_seed("track", A->c[i].name), &nom, d);
        spread_of(nom, d, k, &s);
        double *o = A->ps + 6 * (size_t)i;
        o[0] = nom.pos.x; o[1] = nom.pos.y; o[2] = nom.pos.z; o[3] = nom.vel.x; o[4] = nom.vel.y; o[5] = nom.vel.z;
        A->sig[2 * (size_t)i] = s.sig_pos;
        A->sig[2 * (size_t)i + 1] = s.sig_vel;
    }
}

void pgh_track_starts(const PhTarget *t, const PhCluster *c, int n, int threads, double *ps, double *sig) {
    StartArg A = {t, t ? NULL : c, ps, sig};
    pgh_parallel_for(n, threads, 16, starts_range, &A);
}

void ph_track_free(PhTrack *t) { free(t->pos); t->pos = NULL; t->n = 0; }

static double nearest_on_segment(V3 r0, V3 r1, double *s_out) {
    V3 dr = sub3(r1, r0);
    double dd = dot3(dr, dr), s = 0;
    if (dd > 0) {
        s = -dot3(r0, dr) / dd;
        if (s < 0) s = 0; else if (s > 1) s = 1;
    }
    *s_out = s;
    return len3(add3(r0, mul3(dr, s)));
}

int ph_prefilter(const PhTrack *tt, const PhTrack *ct, const PhCluster *c) {
    int n = tt->n < ct->n ? tt->n : ct->n;
    double sp = hypot(tt->sig_pos, ct->sig_pos), sv = hypot(tt->sig_vel, ct->sig_vel);
    double r0 = (3.0 * c->rtot_pc + 10.0) / 1000.0;
    for (int k = 0; k + 1 < n; k++) {
        double s, d = nearest_on_segment(sub3(fromv(tt->pos[k]), fromv(ct->pos[k])),
                                         sub3(fromv(tt->pos[k + 1]), fromv(ct->pos[k + 1])), &s);
        if (d < r0 + 3.0 * (sp + sv * ((k + s) * PH_PRE_STEP_MYR))) return 1;
    }
    return 0;
}

/* ---- seeds --------------------------------------------------------------------------------------------------- */
uint64_t pgh_fnv_continue(uint64_t h, const char *s) {
    for (const unsigned char *p = (const unsigned char *)s; *p; p++) h = (h ^ *p) * 1099511628211ULL;
    return h;
}
uint64_t pgh_seed_prefix(const char *target_id) {     /* FNV-1a state after "target_id|" */
    uint64_t h = pgh_fnv_continue(1469598103934665603ULL, target_id);
    return (h ^ (unsigned char)'|') * 1099511628211ULL;
}
uint64_t ph_seed(const char *a, const char *b) { return pgh_fnv_continue(pgh_seed_prefix(a), b); }

/* ---- readers ------------------------------------------------------------------------------------------------ */
static double num_or_nan(const char *s) { return strcmp(s, "nan") == 0 ? NAN : atof(s); }

int ph_read_clusters(const char *path, PhCluster **out) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    int cap = 1024, n = 0, idx;
    PhCluster *v = malloc(sizeof(PhCluster) * cap);
    char line[1024], a[32], b[32], kind[4];
    while (fgets(line, sizeof line, f)) {
        if (n == cap) { cap *= 2; v = realloc(v, sizeof(PhCluster) * cap); }
        PhCluster *c = &v[n];
        if (sscanf(line, "%d %39s %3s %lf %lf %lf %lf %lf %lf %lf %lf %31s %31s %lf %lf %lf %lf %lf %lf", &idx,
                   c->name, kind, &c->ra, &c->dec, &c->dist_pc, &c->e_dist_pc, &c->pmra, &c->e_pmra, &c->pmdec,
                   &c->e_pmdec, a, b, &c->r50_pc, &c->rtot_pc, &c->age16, &c->age50, &c->age84, &c->tmax_myr) != 19)
            continue;
        c->kind = kind[0];
        c->rv = num_or_nan(a);
        c->e_rv = num_or_nan(b);
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
    char line[1024], a[32], b[32], kind[4];
    while (fgets(line, sizeof line, f)) {
        if (n == cap) { cap *= 2; v = realloc(v, sizeof(PhTarget) * cap); }
        PhTarget *t = &v[n];
        if (sscanf(line, "%39s %3s %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %31s %31s", t->id, kind, &t->ra, &t->dec,
                   &t->plx, &t->e_plx, &t->dist_pc, &t->e_lndist, &t->pmra, &t->e_pmra, &t->pmdec, &t->e_pmdec, a,
                   b) != 14)
            continue;
        t->kind = kind[0];
        t->rv = num_or_nan(a);
        t->e_rv = num_or_nan(b);
        t->has_rv = !isnan(t->rv) && !isnan(t->e_rv);
        n++;
    }
    fclose(f);
    *out = v;
    return n;
}

/* ---- threaded batch draws ------------------------------------------------------------------------------------ */
typedef struct {
    const PhTarget *t;
    const PhCluster *c;
    int n, n_samp, next, chunk;
    double *ps0, *sig;
    uint64_t *prefix;
    pthread_mutex_t mu;
} DrawJob;

static void *draw_worker(void *arg) {
    DrawJob *J = arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int i0 = J->next;
        J->next += J->chunk;
        pthread_mutex_unlock(&J->mu);
        if (i0 >= J->n) return NULL;
        int i1 = i0 + J->chunk < J->n ? i0 + J->chunk : J->n;
        for (int i = i0; i < i1; i++) {
            if (J->t) {
                pgh_target_init(&J->t[i], J->n_samp, ph_seed("lin", J->t[i].id), J->ps0 + 6 * (size_t)i,
                                J->sig + 36 * (size_t)i);
                if (J->prefix) J->prefix[i] = pgh_seed_prefix(J->t[i].id);
            } else {
                pgh_cluster_init(&J->c[i], J->n_samp, ph_seed("lin", J->c[i].name), J->ps0 + 6 * (size_t)i,
                                 J->sig + 36 * (size_t)i);
            }
        }
    }
}

static void run_draws(DrawJob *J, int threads) {
    ensure_init();
    pthread_mutex_init(&J->mu, NULL);
    J->next = 0;
    J->chunk = 16;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if (threads == 1 || J->n < 64) {
        draw_worker(J);
    } else {
        pthread_t th[256];
        int started = 0;
        for (int i = 0; i < threads; i++) if (pthread_create(&th[started], NULL, draw_worker, J) == 0) started++;
        if (started == 0) draw_worker(J);
        for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
    }
    pthread_mutex_destroy(&J->mu);
}

void pgh_draw_targets(const PhTarget *t, int n, int n_samp, int threads, double *ps0, double *sig, uint64_t *prefix) {
    DrawJob J;
    memset(&J, 0, sizeof J);
    J.t = t; J.n = n; J.n_samp = n_samp; J.ps0 = ps0; J.sig = sig; J.prefix = prefix;
    run_draws(&J, threads);
}

void pgh_draw_clusters(const PhCluster *c, int n, int n_samp, int threads, double *ps0, double *sig) {
    DrawJob J;
    memset(&J, 0, sizeof J);
    J.c = c; J.n = n; J.n_samp = n_samp; J.ps0 = ps0; J.sig = sig;
    run_draws(&J, threads);
}

int pgh_default_threads(void) {
    const char *e = getenv("PHYGAS_HOST_THREADS");
    int n = e ? atoi(e) : 0;
    if (n > 0) return n;
#ifdef _SC_NPROCESSORS_ONLN
    n = (int)sysconf(_SC_NPROCESSORS_ONLN);
#endif
    return n > 0 ? n : 8;
}

/* ---- host parallel loop and batched pair draws ------------------------------------------------------------- */
typedef struct {
    int n, next, chunk;
    void (*fn)(void *, int, int);
    void *arg;
    pthread_mutex_t mu;
} ForJob;

static void *for_worker(void *p) {
    ForJob *J = p;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int i0 = J->next;
        J->next += J->chunk;
        pthread_mutex_unlock(&J->mu);
        if (i0 >= J->n) return NULL;
        J->fn(J->arg, i0, i0 + J->chunk < J->n ? i0 + J->chunk : J->n);
    }
}

void pgh_parallel_for(int n, int threads, int chunk, void (*fn)(void *, int, int), void *arg) {
    ForJob J;
    ensure_init();
    J.n = n; J.next = 0; J.chunk = chunk > 0 ? chunk : 1; J.fn = fn; J.arg = arg;
    pthread_mutex_init(&J.mu, NULL);
    if (threads > 256) threads = 256;
    if (threads <= 1 || n <= J.chunk) {
        for_worker(&J);
    } else {
        pthread_t th[256];
        int started = 0;
        for (int i = 0; i < threads; i++) if (pthread_create(&th[started], NULL, for_worker, &J) == 0) started++;
        if (started == 0) for_worker(&J);
        for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
    }
    pthread_mutex_destroy(&J.mu);
}

typedef struct {
    const PhTarget *const *t;
    const PhCluster *const *c;
    int n_clones;
    double dt_myr;
    const uint64_t *seed;
    double *ps;
    int *m, *steps;
    double *dt;
} PairDrawArg;

static void pair_draw_range(void *p, int i0, int i1) {
    PairDrawArg *A = p;
    for (int i = i0; i < i1; i++)
        A->m[i] = ph_pair_draw(A->t[i], A->c[i], A->n_clones, A->dt_myr, A->seed[i],
                               A->ps + (size_t)i * 12 * A->n_clones, &A->steps[i], &A->dt[i]);
}

void pgh_draw_pairs(int n_pairs, const PhTarget *const *t, const PhCluster *const *c, int n_clones, double dt_myr,
                    const uint64_t *seed, int threads, double *ps, int *m, int *steps, double *dt) {
    PairDrawArg A = {t, c, n_clones, dt_myr, seed, ps, m, steps, dt};
    pgh_parallel_for(n_pairs, threads, 4, pair_draw_range, &A);
}

/* ---- batched pair jobs: tracks + prefilter, and clone draws with a clone count per pair ------------------------ */
typedef struct {
    const PhCluster *c;
    PhTrack *tr;
} ClusterTrackArg;

static void cluster_track_range(void *p, int i0, int i1) {
    ClusterTrackArg *A = p;
    for (int i = i0; i < i1; i++) ph_track_cluster(&A->c[i], 32, ph_seed("track", A->c[i].name), &A->tr[i]);
}

typedef struct {
    const PhTarget *t;
    const PhCluster *c;
    const PhTrack *ctr;
    int nc;
    double tmax;
    unsigned char *keep;      /* [nt][nc] */
} PrefilterArg;

static void prefilter_range(void *p, int j0, int j1) {
    PrefilterArg *A = p;
    for (int j = j0; j < j1; j++) {
        PhTrack tt;
        ph_track_target(&A->t[j], A->tmax, 32, ph_seed("track", A->t[j].id), &tt);
        unsigned char *k = A->keep + (size_t)j * A->nc;
        for (int i = 0; i < A->nc; i++) k[i] = (unsigned char)ph_prefilter(&tt, &A->ctr[i], &A->c[i]);
        ph_track_free(&tt);
    }
}

long pgh_prefilter_pairs(const PhTarget *t, int nt, const PhCluster *c, int nc, int threads, int *ti, int *ci,
                         long cap) {
    if (nt <= 0 || nc <= 0) return 0;
    double tmax = 0;
    for (int i = 0; i < nc; i++) if (c[i].tmax_myr > tmax) tmax = c[i].tmax_myr;
    PhTrack *ctr = malloc(sizeof(PhTrack) * (size_t)nc);
    unsigned char *keep = malloc((size_t)nt * nc);
    if (!ctr || !keep) { free(ctr); free(keep); return -1; }
    ClusterTrackArg ca = {c, ctr};
    pgh_parallel_for(nc, threads, 16, cluster_track_range, &ca);
    PrefilterArg pa = {t, c, ctr, nc, tmax, keep};
    pgh_parallel_for(nt, threads, 1, prefilter_range, &pa);
    long n = 0;
    for (int j = 0; j < nt; j++)
        for (int i = 0; i < nc; i++) {
            if (!keep[(size_t)j * nc + i]) continue;
            if (n < cap) { ti[n] = j; ci[n] = i; }
            n++;
        }
    for (int i = 0; i < nc; i++) ph_track_free(&ctr[i]);
    free(ctr);
    free(keep);
    return n;
}

typedef struct {
    const PhTarget *t;
    const int *ti;
    const PhCluster *c;
    const int *ci;
    const int *n_clones;
    const long *slot;         /* first clone slot of pair q, before compaction */
    double dt_myr;
    double *ps;
    int *m, *steps;
    double *dt;
} BatchDrawArg;

static void batch_draw_range(void *p, int q0, int q1) {
    BatchDrawArg *A = p;
    for (int q = q0; q < q1; q++) {
        const PhTarget *t = &A->t[A->ti[q]];
        const PhCluster *c = &A->c[A->ci[q]];
        A->m[q] = ph_pair_draw(t, c, A->n_clones[q], A->dt_myr, ph_seed(t->id, c->name), A->ps + 12 * A->slot[q],
                               &A->steps[q], &A->dt[q]);
    }
}

int pgh_draw_pair_batch(int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c, const int *ci,
                        const int *n_clones, double dt_myr, int threads, int *clone_off, double *ps, int *steps,
                        double *dt, double *r50_pc, double *rtot_pc) {
    long *slot = malloc(sizeof(long) * (size_t)(n_pairs + 1));
    int *m = malloc(sizeof(int) * (size_t)(n_pairs > 0 ? n_pairs : 1));
    if (!slot || !m) { free(slot); free(m); return -1; }
    slot[0] = 0;
    for (int q = 0; q < n_pairs; q++) slot[q + 1] = slot[q] + (n_clones[q] > 0 ? n_clones[q] : 0);
    BatchDrawArg A = {t, ti, c, ci, n_clones, slot, dt_myr, ps, m, steps, dt};
    pgh_parallel_for(n_pairs, threads, 4, batch_draw_range, &A);
    /* compact: the clones of pair q follow those of pair q - 1 (a pair keeps only its successful draws) */
    long off = 0;
    clone_off[0] = 0;
    for (int q = 0; q < n_pairs; q++) {
        if (off != slot[q] && m[q] > 0) memmove(ps + 12 * off, ps + 12 * slot[q], sizeof(double) * 12 * (size_t)m[q]);
        off += m[q];
        if (off > 2147483647L) { free(slot); free(m); return -2; }
        clone_off[q + 1] = (int)off;
        r50_pc[q] = c[ci[q]].r50_pc;
        rtot_pc[q] = c[ci[q]].rtot_pc;
    }
    free(slot);
    free(m);
    return 0;
}

/* the chance-alignment control of the screen (reference phygas_screen.c:35-47): star j takes the proper motions of
 * the star n/2 further on (cyclically), rescaled by the parallax ratio, and its radial velocity */
void pgh_control_targets(const PhTarget *t, int n, PhTarget *out) {
    for (int j = 0; j < n; j++) {
        out[j] = t[j];
        const PhTarget *o = &t[(j + n / 2) % n];
        double f = (t[j].plx > 0 && o->plx > 0) ? t[j].plx / o->plx : 1.0;
        out[j].pmra = o->pmra * f; out[j].e_pmra = o->e_pmra * f;
        out[j].pmdec = o->pmdec * f; out[j].e_pmdec = o->e_pmdec * f;
        out[j].rv = o->rv; out[j].e_rv = o->e_rv; out[j].has_rv = o->has_rv;
    }
}
