/* phygas.h -- drop-in C API of the Phygas orbit hot paths, served by libphygas_gb300.
 *
 * A program written against the reference's `src/phygas.h` compiles against this header and links against
 * libphygas_gb300.so unchanged: the record types keep their field order and meaning (the ABI), and every function
 * keeps its name, arguments, ownership rule and error behaviour.  Behind them the orbit integration, the chi2 scan,
 * the 512-draw probabilities and the clone Monte Carlo run as CUDA kernels on the GPU (see phygas_gb300.h for the
 * batched entry points these wrappers call).  The draws from measurement errors, the seeds and the file readers run
 * on the host, as in the reference's GPU application.
 *
 * Units inside: kpc, Myr, kpc/Myr.  Reported: pc, Myr (positive = in the past), km/s.
 *
 * Each declaration names the reference declaration it replaces (path:line within the reference project).
 */
#ifndef PHYGAS_H
#define PHYGAS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- small records shared with the orbit core (reference src/vec3.h:6, src/coords.h:22-51,
 *      src/montecarlo.h:22-24, src/potential.h:13-19, src/potential.h:73-85) ------------------------------- */
typedef struct { double x, y, z; } Vec3;                       /* src/vec3.h:6 */

typedef struct {                                               /* src/coords.h:22-29 */
    double ra_deg, dec_deg;      /* ICRS, degrees */
    double parallax_mas;         /* > 0 */
    double pmra_masyr;           /* includes cos(dec) */
    double pmdec_masyr;
    double rv_kms;
} Astrometry;

typedef struct { Vec3 pos; Vec3 vel; } PhaseSpace;             /* src/coords.h:31-34; kpc, kpc/Myr */

typedef struct {                                               /* src/coords.h:42-49 */
    double r0_kpc, z0_kpc, v_circ_kms, u_pec_kms, v_pec_kms, w_pec_kms;
} SolarParams;

typedef struct { uint64_t state; } McRng;                      /* src/montecarlo.h:22-24 (splitmix64 state) */

typedef struct Potential Potential;                            /* src/potential.h:13-19 */
struct Potential {
    void (*acceleration)(const Potential *pot, Vec3 pos, Vec3 *accel_out);
    double (*energy)(const Potential *pot, Vec3 pos);
    const void *params;
};

typedef struct {                                               /* src/potential.h:73-83 */
    double bulge_GM, bulge_b;                  /* Plummer bulge */
    double disk_GM, disk_a, disk_b;            /* Miyamoto-Nagai disk */
    double halo_GM, halo_a, halo_cutoff, halo_gamma;   /* truncated Allen & Santillan halo */
} MilkyWayParams;

extern const MilkyWayParams milkyway_potential_default;        /* src/potential.h:85 */
extern const SolarParams solar_params_default;                 /* src/coords.h:51 */

/* ---- input records and results (reference src/phygas.h:19-57) ------------------------------------------------ */
typedef struct {                                               /* src/phygas.h:19-30 */
    char name[40];
    char kind;                   /* o = open cluster, m = moving group */
    double ra, dec;
    double dist_pc, e_dist_pc;
    double pmra, e_pmra, pmdec, e_pmdec;
    double rv, e_rv;
    int has_rv;                  /* 0: drawn around the Galactic-rotation expectation +- PH_CLUSTER_RV_PRIOR */
    double r50_pc, rtot_pc;
    double age16, age50, age84;
    double tmax_myr;
} PhCluster;

typedef struct {                                               /* src/phygas.h:32-41 */
    char id[40];
    char kind;                   /* P = pulsar / neutron star, S = star */
    double ra, dec;
    double plx, e_plx;           /* used when plx > 0 */
    double dist_pc, e_lndist;    /* used when plx == 0: log-normal distance */
    double pmra, e_pmra, pmdec, e_pmdec;
    double rv, e_rv;
    int has_rv;
} PhTarget;

typedef struct {                                               /* src/phygas.h:44-49 */
    int n;
    Vec3 *pos;
    double sig_pos;
    double sig_vel;
} PhTrack;

typedef struct {                                               /* src/phygas.h:51-57 */
    int n;
    double d05, d50, d95;
    double t05, t50, t95;
    double v05, v50, v95;
    double f_r50, f_rtot;
} PhResult;

typedef struct {                                               /* src/phygas.h:100-104 */
    int n;
    Vec3 *pos, *vel;
    double (*S)[6];              /* xx xy xz yy yz zz, kpc^2 */
} PhLin;

typedef struct {                                               /* src/phygas.h:106-113 */
    double chi2;
    double t;
    double d_nom_pc;
    double sig_pc;
    double p_r50, p_rtot;
    double vrel;
} PhScreen;

#define PH_PRE_STEP_MYR 0.5           /* src/phygas.h:59 */
#define PH_CLUSTER_RV_PRIOR 10.0      /* src/phygas.h:60 */
#define PH_PULSAR_RV_PRIOR 265.0      /* src/phygas.h:61 */
#define PH_STAR_RV_PRIOR 30.0         /* src/phygas.h:62 */
#define PH_LIN_EPS_POS 1e-5           /* src/phygas.h:119 */
#define PH_LIN_EPS_VEL 1e-5           /* src/phygas.h:120 */
#define PH_LIN_SUB 10                 /* src/phygas.h:121 */

/* ---- entry points (reference src/phygas.h:64-139) -------------------------------------------------------------- */
void ph_init(void);                                                                     /* src/phygas.h:64 */
const Potential *ph_potential(void);                                                    /* src/phygas.h:65 */

int ph_sample_target(const PhTarget *t, McRng *rng, PhaseSpace *out);                   /* src/phygas.h:68 */
int ph_sample_cluster(const PhCluster *c, McRng *rng, PhaseSpace *out);                 /* src/phygas.h:69 */

void ph_track_target(const PhTarget *t, double tmax_myr, int n_spread, uint64_t seed, PhTrack *out); /* :72 */
void ph_track_cluster(const PhCluster *c, int n_spread, uint64_t seed, PhTrack *out);               /* :73 */
void ph_track_free(PhTrack *t);                                                                       /* :74 */
int ph_prefilter(const PhTrack *target, const PhTrack *cluster, const PhCluster *c);                 /* :78 */

void ph_pair(const PhTarget *t, const PhCluster *c, int n_clones, double dt_myr, uint64_t seed,
             PhResult *res);                                                                         /* :81 */
int ph_pair_draw(const PhTarget *t, const PhCluster *c, int n_clones, double dt_myr, uint64_t seed,
                 double *ps, int *steps, double *dt);                                                /* :87 */
void ph_pair_clone(const double *ps, int steps, double dt, double *best, double *tbest, double *vbest); /* :89 */
void ph_pair_reduce(const PhCluster *c, int m, const double *best, const double *tbest, const double *vbest,
                    PhResult *res);                                                                  /* :90 */

void ph_lin_target(const PhTarget *t, double tmax_myr, int n_samp, uint64_t seed, PhLin *out);       /* :115 */
void ph_lin_target_init(const PhTarget *t, int n_samp, uint64_t seed, double ps0[6], double sig[6][6]); /* :118 */
void ph_lin_cluster(const PhCluster *c, int n_samp, uint64_t seed, PhLin *out);                      /* :122 */
void ph_lin_free(PhLin *l);                                                                          /* :123 */
extern double ph_screen_r;                                                                           /* :124 */
void ph_screen(const PhLin *t, const PhLin *c, const PhCluster *cl, uint64_t seed, PhScreen *res);   /* :125 */
double ph_screen_chi2(const PhLin *t, const PhLin *c, const PhCluster *cl, int *kb, double *sb);     /* :128 */
double ph_screen_chi2_cut(const PhLin *t, const PhLin *c, const PhCluster *cl, double chi2_max, int *kb,
                          double *sb);                                                               /* :131 */
void ph_screen_finish(const PhLin *t, const PhLin *c, const PhCluster *cl, uint64_t seed, double chi2,
                      int kb, double sb, PhScreen *res);                                             /* :132 */

uint64_t ph_seed(const char *target_id, const char *cluster_name);                                  /* :135 */

int ph_read_clusters(const char *path, PhCluster **out);                                            /* :138 */
int ph_read_targets(const char *path, PhTarget **out);                                              /* :139 */

#ifdef __cplusplus
}
#endif
#endif
