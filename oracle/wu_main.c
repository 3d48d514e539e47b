/* wu_main.c -- work-unit runner over the reference C API (test infrastructure).
 *
 * Prints the result rows a Phygas work unit produces (the row formats and loop order of the reference BOINC app's CPU
 * loop, src/main_phygas_boinc.cpp:431-456), for a slice of it, so that a test can run slices in parallel and hash the
 * concatenation against the reference's published row hashes (docs/BENCHMARK.md:366).  Linked against the oracle.
 *
 * usage: wu clusters in [j0 j1 [i0 i1]]
 *   in: line 1 "PHYGAS 1 screen <chi2_max> <n_samp> <r_kernel> <p_min>" or "PHYGAS 1 pair <n_clones> <dt_myr>",
 *       then one target per line (14 fields, optionally "clusters=NAME,...").
 *   Rows of targets [j0,j1) against clusters [i0,i1), in (target, cluster) order.  No "# done" line.
 *   stderr: "wu_time prep <s> run <s>" -- the per-cluster precompute and the per-target loop, timed apart.
 *   With PHYGAS_WU_RAW set in the environment, screen mode writes each kept pair to stdout as one binary record
 *   instead of the text row, so a caller can compare the values at full precision: int32 target index, cluster
 *   index, kb, 0, then doubles sb, chi2, t, d_nom_pc, sig_pc, p_r50, p_rtot, vrel (80 bytes, host byte order; the
 *   layout of PgxScreenRow in include/phygas_gb300.h).
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "phygas.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + ts.tv_nsec * 1e-9;
}

static int listed(const char *name, const char *list) {
    size_t n = strlen(name);
    for (const char *p = list; (p = strstr(p, name)) != NULL; p += n)
        if ((p == list || p[-1] == ',') && (p[n] == ',' || p[n] == '\0')) return 1;
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 3) { fprintf(stderr, "usage: wu clusters in [j0 j1 [i0 i1]]\n"); return 2; }
    ph_init();
    PhCluster *cl;
    int nc = ph_read_clusters(argv[1], &cl);
    FILE *f = fopen(argv[2], "r");
    if (nc <= 0 || !f) { fprintf(stderr, "can't read inputs\n"); return 1; }
    static char line[65536];
    char mode[16] = "";
    double p1 = 0, p2 = 0, p3 = 0, p4 = 0;
    if (!fgets(line, sizeof line, f) || sscanf(line, "PHYGAS 1 %15s %lf %lf %lf %lf", mode, &p1, &p2, &p3, &p4) < 3) {
        fprintf(stderr, "bad header\n");
        return 1;
    }
    int cap = 1024, nt = 0;
    PhTarget *tg = malloc(sizeof(PhTarget) * cap);
    char **only = malloc(sizeof(char *) * cap);
    while (fgets(line, sizeof line, f)) {
        if (nt == cap) { cap *= 2; tg = realloc(tg, sizeof(PhTarget) * cap); only = realloc(only, sizeof(char *) * cap); }
        PhTarget *t = &tg[nt];
        char srv[32], serv[32], kind[4];
        int used = 0;
        if (sscanf(line, "%39s %3s %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %31s %31s%n", t->id, kind, &t->ra, &t->dec,
                   &t->plx, &t->e_plx, &t->dist_pc, &t->e_lndist, &t->pmra, &t->e_pmra, &t->pmdec, &t->e_pmdec, srv,
                   serv, &used) != 14)
            continue;
        t->kind = kind[0];
        t->rv = strcmp(srv, "nan") ? atof(srv) : NAN;
        t->e_rv = strcmp(serv, "nan") ? atof(serv) : NAN;
        t->has_rv = !isnan(t->rv) && !isnan(t->e_rv);
        only[nt] = NULL;
        const char *p = strstr(line + used, "clusters=");
        if (p) {   /* an empty list is no list: the prefilter decides (reference main_phygas_boinc.cpp:318-321, 393) */
            size_t len = strcspn(p + 9, " \r\n");
            if (len > 0) {
                only[nt] = malloc(len + 1);
                memcpy(only[nt], p + 9, len);
                only[nt][len] = 0;
            }
        }
        nt++;
    }
    fclose(f);
    int j0 = argc > 3 ? atoi(argv[3]) : 0, j1 = argc > 4 ? atoi(argv[4]) : nt;
    int i0 = argc > 5 ? atoi(argv[5]) : 0, i1 = argc > 6 ? atoi(argv[6]) : nc;
    if (j1 > nt) j1 = nt;
    if (i1 > nc) i1 = nc;
    double tmax = 0;
    for (int i = 0; i < nc; i++) if (cl[i].tmax_myr > tmax) tmax = cl[i].tmax_myr;
    const int raw = getenv("PHYGAS_WU_RAW") != NULL;
    double t_prep = 0, t_run = 0, t0 = now_s();
    if (!strcmp(mode, "screen")) {
        ph_screen_r = p3 > 0 ? p3 : 2.0;
        PhLin *cin = calloc(nc, sizeof(PhLin));
        for (int i = i0; i < i1; i++) ph_lin_cluster(&cl[i], (int)p2, ph_seed("lin", cl[i].name), &cin[i]);
        t_prep = now_s() - t0;
        t0 = now_s();
        for (int j = j0; j < j1; j++) {
            PhLin tl;
            ph_lin_target(&tg[j], tmax, (int)p2, ph_seed("lin", tg[j].id), &tl);
            for (int i = i0; i < i1; i++) {
                int kb;
                double sb, chi2 = ph_screen_chi2_cut(&tl, &cin[i], &cl[i], p1, &kb, &sb);
                if (!(chi2 < p1)) continue;
                PhScreen s;
                ph_screen_finish(&tl, &cin[i], &cl[i], ph_seed(tg[j].id, cl[i].name), chi2, kb, sb, &s);
                if (s.p_r50 < p4) continue;
                if (raw) {
                    struct { int j, i, kb, pad; double v[8]; } rec = {j, i, kb, 0, {sb, s.chi2, s.t, s.d_nom_pc,
                                                                                    s.sig_pc, s.p_r50, s.p_rtot,
                                                                                    s.vrel}};
                    fwrite(&rec, sizeof rec, 1, stdout);
                } else
                    printf("%s %s %c %.3f %.3f %.2f %.2f %.4f %.4f %.2f\n", tg[j].id, cl[i].name, cl[i].kind, s.chi2,
                           s.t, s.d_nom_pc, s.sig_pc, s.p_r50, s.p_rtot, s.vrel);
            }
            ph_lin_free(&tl);
        }
    } else if (!strcmp(mode, "pair")) {
        PhTrack *ctr = calloc(nc, sizeof(PhTrack));
        for (int i = i0; i < i1; i++) ph_track_cluster(&cl[i], 32, ph_seed("track", cl[i].name), &ctr[i]);
        t_prep = now_s() - t0;
        t0 = now_s();
        for (int j = j0; j < j1; j++) {
            PhTrack tt;
            ph_track_target(&tg[j], tmax, 32, ph_seed("track", tg[j].id), &tt);
            for (int i = i0; i < i1; i++) {
                if (only[j] ? !listed(cl[i].name, only[j]) : !ph_prefilter(&tt, &ctr[i], &cl[i])) continue;
                PhResult r;
                ph_pair(&tg[j], &cl[i], (int)p1, p2, ph_seed(tg[j].id, cl[i].name), &r);
                printf("%s %s %c %d %.3f %.3f %.3f %.4f %.4f %.4f %.2f %.2f %.2f %.4f %.4f\n", tg[j].id, cl[i].name,
                       cl[i].kind, r.n, r.d05, r.d50, r.d95, r.t05, r.t50, r.t95, r.v05, r.v50, r.v95, r.f_r50,
                       r.f_rtot);
            }
            ph_track_free(&tt);
        }
    } else {
        fprintf(stderr, "unknown mode %s\n", mode);
        return 1;
    }
    t_run = now_s() - t0;
    fflush(stdout);
    fprintf(stderr, "wu_time prep %.6f run %.6f\n", t_prep, t_run);
    return 0;
}
