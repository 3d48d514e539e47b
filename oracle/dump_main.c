/* dump_main.c -- raw-value dump harness over the reference C API (test infrastructure).
 *
 * Built twice by oracle/Makefile: against the reference core compiled from its own sources (_ref/ref_dump) and
 * against the oracle restatement (_build/oracle_dump).  Both print every double as a C99 hex float (%a), so the two
 * outputs are compared byte for byte: that comparison is what pins the oracle to the reference.
 *
 * usage:
 *   dump draws  clusters targets j0 j1 n_samp            ph_lin_target_init of targets [j0,j1)
 *   dump lin    clusters targets c|t i0 i1 n_samp         ph_lin_cluster / ph_lin_target (tmax = max cluster tmax)
 *   dump screen clusters targets j0 j1 chi2_max n_samp r_kernel   ph_screen_chi2_cut + ph_screen_finish, kept pairs
 *   dump chi2   clusters targets j0 j1 n_samp r_kernel     ph_screen_chi2 of every pair (no cut)
 *   dump pair   clusters targets j i0 i1 n_clones dt_myr   ph_pair_draw / ph_pair_clone / ph_pair_reduce, no prefilter
 *   dump track  clusters targets j n_spread                ph_track_target / ph_track_cluster / ph_prefilter
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "phygas.h"

static PhCluster *cl;
static PhTarget *tg;
static int nc, nt;

static double max_tmax(void) {
    double t = 0;
    for (int i = 0; i < nc; i++) if (cl[i].tmax_myr > t) t = cl[i].tmax_myr;
    return t;
}

static void put_lin(const char *tag, int id, const PhLin *l) {
    for (int k = 0; k < l->n; k++)
        printf("%s %d %d %a %a %a %a %a %a %a %a %a %a %a %a\n", tag, id, k, l->pos[k].x, l->pos[k].y, l->pos[k].z,
               l->vel[k].x, l->vel[k].y, l->vel[k].z, l->S[k][0], l->S[k][1], l->S[k][2], l->S[k][3], l->S[k][4],
               l->S[k][5]);
}

int main(int argc, char **argv) {
    if (argc < 4) { fprintf(stderr, "usage: see dump_main.c\n"); return 2; }
    const char *mode = argv[1];
    ph_init();
    nc = ph_read_clusters(argv[2], &cl);
    nt = ph_read_targets(argv[3], &tg);
    if (nc <= 0 || nt <= 0) { fprintf(stderr, "can't read inputs\n"); return 1; }
    if (!strcmp(mode, "draws")) {
        int j0 = atoi(argv[4]), j1 = atoi(argv[5]), ns = atoi(argv[6]);
        for (int j = j0; j < j1 && j < nt; j++) {
            double ps0[6], sig[6][6];
            ph_lin_target_init(&tg[j], ns, ph_seed("lin", tg[j].id), ps0, sig);
            printf("ps0 %d", j);
            for (int i = 0; i < 6; i++) printf(" %a", ps0[i]);
            printf("\nsig %d", j);
            for (int a = 0; a < 6; a++) for (int b = 0; b < 6; b++) printf(" %a", sig[a][b]);
            printf("\n");
        }
    } else if (!strcmp(mode, "lin")) {
        char which = argv[4][0];
        int i0 = atoi(argv[5]), i1 = atoi(argv[6]), ns = atoi(argv[7]);
        double tmax = max_tmax();
        for (int i = i0; i < i1; i++) {
            PhLin l;
            if (which == 'c') {
                if (i >= nc) break;
                ph_lin_cluster(&cl[i], ns, ph_seed("lin", cl[i].name), &l);
            } else {
                if (i >= nt) break;
                ph_lin_target(&tg[i], tmax, ns, ph_seed("lin", tg[i].id), &l);
            }
            put_lin(which == 'c' ? "c" : "t", i, &l);
            ph_lin_free(&l);
        }
    } else if (!strcmp(mode, "screen") || !strcmp(mode, "chi2")) {
        int cut_mode = !strcmp(mode, "screen");
        int j0 = atoi(argv[4]), j1 = atoi(argv[5]);
        double cut = cut_mode ? atof(argv[6]) : 0;
        int ns = atoi(argv[cut_mode ? 7 : 6]);
        ph_screen_r = atof(argv[cut_mode ? 8 : 7]);
        double tmax = max_tmax();
        PhLin *cin = malloc(sizeof(PhLin) * nc);
        for (int i = 0; i < nc; i++) ph_lin_cluster(&cl[i], ns, ph_seed("lin", cl[i].name), &cin[i]);
        for (int j = j0; j < j1 && j < nt; j++) {
            PhLin tl;
            ph_lin_target(&tg[j], tmax, ns, ph_seed("lin", tg[j].id), &tl);
            for (int i = 0; i < nc; i++) {
                int kb;
                double sb;
                if (cut_mode) {
                    double chi2 = ph_screen_chi2_cut(&tl, &cin[i], &cl[i], cut, &kb, &sb);
                    if (!(chi2 < cut)) continue;
                    PhScreen s;
                    ph_screen_finish(&tl, &cin[i], &cl[i], ph_seed(tg[j].id, cl[i].name), chi2, kb, sb, &s);
                    printf("%d %d %a %d %a %a %a %a %a %a %a\n", j, i, s.chi2, kb, sb, s.t, s.d_nom_pc, s.sig_pc,
                           s.p_r50, s.p_rtot, s.vrel);
                } else {
                    double chi2 = ph_screen_chi2(&tl, &cin[i], &cl[i], &kb, &sb);
                    printf("%d %d %a %d %a\n", j, i, chi2, kb, sb);
                }
            }
            ph_lin_free(&tl);
        }
        for (int i = 0; i < nc; i++) ph_lin_free(&cin[i]);
        free(cin);
    } else if (!strcmp(mode, "pair")) {
        int j = atoi(argv[4]), i0 = atoi(argv[5]), i1 = atoi(argv[6]), n = atoi(argv[7]);
        double dtm = atof(argv[8]);
        double *ps = malloc(sizeof(double) * 12 * (n > 0 ? n : 1)), *r = malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
        for (int i = i0; i < i1 && i < nc; i++) {
            int steps;
            double dt;
            int m = ph_pair_draw(&tg[j], &cl[i], n, dtm, ph_seed(tg[j].id, cl[i].name), ps, &steps, &dt);
            printf("draw %d %d %d %d %a\n", j, i, m, steps, dt);
            for (int k = 0; k < m; k++) {
                printf("ps %d", k);
                for (int c = 0; c < 12; c++) printf(" %a", ps[12 * k + c]);
                printf("\n");
                ph_pair_clone(ps + 12 * k, steps, dt, &r[k], &r[m + k], &r[2 * m + k]);
                printf("clone %d %a %a %a\n", k, r[k], r[m + k], r[2 * m + k]);
            }
            PhResult res;
            ph_pair_reduce(&cl[i], m, r, r + m, r + 2 * m, &res);
            printf("res %d %d %d %a %a %a %a %a %a %a %a %a %a %a\n", j, i, res.n, res.d05, res.d50, res.d95, res.t05,
                   res.t50, res.t95, res.v05, res.v50, res.v95, res.f_r50, res.f_rtot);
        }
        free(ps);
        free(r);
    } else if (!strcmp(mode, "track")) {
        int j = atoi(argv[4]), nsp = atoi(argv[5]);
        PhTrack tt;
        ph_track_target(&tg[j], max_tmax(), nsp, ph_seed("track", tg[j].id), &tt);
        printf("target %d %d %a %a\n", j, tt.n, tt.sig_pos, tt.sig_vel);
        for (int k = 0; k < tt.n; k++) printf("tp %d %a %a %a\n", k, tt.pos[k].x, tt.pos[k].y, tt.pos[k].z);
        for (int i = 0; i < nc; i++) {
            PhTrack ct;
            ph_track_cluster(&cl[i], nsp, ph_seed("track", cl[i].name), &ct);
            printf("cluster %d %d %a %a %d\n", i, ct.n, ct.sig_pos, ct.sig_vel, ph_prefilter(&tt, &ct, &cl[i]));
            ph_track_free(&ct);
        }
        ph_track_free(&tt);
    } else {
        fprintf(stderr, "unknown mode %s\n", mode);
        return 2;
    }
    return 0;
}
