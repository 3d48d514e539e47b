/* phygas_screen -- drop-in for the reference's stage-1 screening CLI (src/phygas_screen.c), on the GPU.
 *
 *   phygas_screen clusters.txt stars.txt [chi2_max=25] [n_samp=64] [r_kernel=2 (x r50; 0 = total radius)] [control]
 *
 * Same arguments, same stdout rows in the same order (star, then cluster; every pair with chi2 < chi2_max):
 *   target cluster kind chi2 t_myr d_nom_pc sig_pc p_r50 p_rtot vrel_kms age16 age84
 * Progress on stderr.  The draws run on all host cores; the orbits, the scan, the 512-draw probabilities and the
 * formatting of the lines on the GPU (libphygas_gb300).  PHYGAS_PRECISION=fp64 selects the plain FP64 screen
 * instead of the default mixed-precision one (their rows are identical); PHYGAS_CHUNK sets the stars per GPU chunk
 * (default 2500: small chunks let the draws, the orbits, the screen and the lines of neighbouring chunks overlap).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "phygas_gb300.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + ts.tv_nsec * 1e-9;
}

typedef struct {
    long kept;
    double t0;
} Printer;

/* one chunk's lines, in (star, cluster) order, formatted on the GPU (pgx_screen_chunks_text) */
static int print_text(void *arg, int first, const char *text, size_t bytes, long n) {
    Printer *P = arg;
    if (bytes && fwrite(text, 1, bytes, stdout) != bytes) return 1;
    P->kept += n;
    fprintf(stderr, "%d+ targets, %ld pairs kept, %.1f s\n", first, P->kept, now_s() - P->t0);
    return 0;
}

static int env_int(const char *name, int def) {
    const char *v = getenv(name);
    int x = v ? atoi(v) : 0;
    return x > 0 ? x : def;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s clusters.txt stars.txt [chi2_max] [n_samp] [r_kernel] [control]\n", argv[0]);
        return 1;
    }
    double chi2_max = argc > 3 ? atof(argv[3]) : 25.0;
    int n_samp = argc > 4 ? atoi(argv[4]) : 64;
    if (argc > 5) ph_screen_r = atof(argv[5]);
    int control = argc > 6 && argv[6][0] == 'c';
    const char *pe = getenv("PHYGAS_PRECISION");
    int precision = pe && !strcmp(pe, "fp64") ? PGX_FP64 : PGX_MIXED;
    ph_init();
    PhCluster *cl;
    PhTarget *tg;
    int nc = ph_read_clusters(argv[1], &cl), nt = ph_read_targets(argv[2], &tg);
    if (nc <= 0 || nt <= 0) { fprintf(stderr, "can't read inputs (%d clusters, %d targets)\n", nc, nt); return 1; }
    double tmax = 0;
    for (int i = 0; i < nc; i++) if (cl[i].tmax_myr > tmax) tmax = cl[i].tmax_myr;
    PgxContext *ctx;
    int rc = pgx_open(-1, &ctx);
    if (rc) { fprintf(stderr, "phygas_screen: no usable GPU (pgx_open: %d)\n", rc); return 1; }
    double t0 = now_s();
    double *cps0 = malloc(sizeof(double) * 6 * nc), *csig = malloc(sizeof(double) * 36 * nc);
    double *ctm = malloc(sizeof(double) * nc), *cr50 = malloc(sizeof(double) * nc), *crt = malloc(sizeof(double) * nc);
    char *names = calloc(nc, 40);
    pgx_draw_clusters(cl, nc, n_samp, 0, cps0, csig);
    for (int i = 0; i < nc; i++) {
        ctm[i] = cl[i].tmax_myr; cr50[i] = cl[i].r50_pc; crt[i] = cl[i].rtot_pc;
        memcpy(names + 40 * (size_t)i, cl[i].name, 40);
    }
    if (pgx_screen_clusters(ctx, nc, cps0, csig, ctm, cr50, crt, names, ph_screen_r)) {
        fprintf(stderr, "phygas_screen: cluster table: %s\n", pgx_last_error(ctx));
        return 1;
    }
    fprintf(stderr, "%d clusters prepared in %.1f s; %d targets\n", nc, now_s() - t0, nt);
    if (control) {   /* velocities of the star nt/2 away, proper motions rescaled by the parallax ratio */
        PhTarget *v = malloc(sizeof(PhTarget) * nt);
        pgx_control_targets(tg, nt, v);
        free(tg);
        tg = v;
        fprintf(stderr, "control run: velocities taken from the star %d lines away\n", nt / 2);
    }
    const int chunk = env_int("PHYGAS_CHUNK", 2500);
    Printer P = {0, now_s()};
    /* the draws of the next chunk run while the GPU screens this one and the previous chunk's lines are written */
    if (pgx_screen_chunks_text(ctx, tg, nt, cl, nc, chunk, n_samp, 0, tmax, chi2_max, precision, print_text, &P)) {
        fprintf(stderr, "phygas_screen: screen: %s\n", pgx_last_error(ctx));
        return 1;
    }
    pgx_close(ctx);
    return 0;
}
