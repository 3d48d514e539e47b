/* phygas_cli -- drop-in for the reference's pair-mode CLI (src/phygas_cli.c), with the clone Monte Carlo on the GPU.
 *
 *   phygas_cli clusters.txt targets.txt [n_clones=1000] [dt_myr=0.05] [only=ID1,ID2,...]
 *
 * Same arguments; one stdout row per (target, cluster) pair that passes the prefilter, in (target, cluster) order:
 *   target cluster kind n d05 d50 d95 t05 t50 t95 v05 v50 v95 f_r50 f_rtot age16 age84
 * The prefilter runs on the GPU (pgx_prefilter: the same pairs as the reference's tracks and ph_prefilter keep), the
 * clone draws (bit-identical to the reference's) on all host cores; the clones of many pairs and targets are traced
 * and reduced together on the GPU (about PHYGAS_BATCH_CLONES per launch, default 2^20, and at least one pair).  Any
 * clone count up to 2^26 per pair: pairs of more than 16,384 clones take their quantiles by radix selection on the
 * GPU instead of a shared-memory sort, with the same results.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "phygas_gb300.h"
#include "ph_host.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + ts.tv_nsec * 1e-9;
}

static int wanted(const char *id, const char *only) {
    if (!only) return 1;
    size_t n = strlen(id);
    for (const char *p = only; (p = strstr(p, id)) != NULL; p += n)
        if ((p == only || p[-1] == ',') && (p[n] == ',' || p[n] == '\0')) return 1;
    return 0;
}

typedef struct {        /* pairs waiting for the GPU */
    int n, cap;
    int *target, *cluster;
} Pending;

static void push(Pending *P, int j, int i) {
    if (P->n == P->cap) {
        P->cap = P->cap ? 2 * P->cap : 4096;
        P->target = realloc(P->target, sizeof(int) * P->cap);
        P->cluster = realloc(P->cluster, sizeof(int) * P->cap);
    }
    P->target[P->n] = j;
    P->cluster[P->n] = i;
    P->n++;
}

static int flush(PgxContext *ctx, Pending *P, const PhTarget *tg, const PhCluster *cl, int n_clones, double dt_myr,
                 int threads) {
    const int np = P->n;
    if (np == 0) return 0;
    const PhTarget **tp = malloc(sizeof(*tp) * np);
    const PhCluster **cp = malloc(sizeof(*cp) * np);
    uint64_t *seed = malloc(sizeof(uint64_t) * np);
    for (int q = 0; q < np; q++) {
        tp[q] = &tg[P->target[q]];
        cp[q] = &cl[P->cluster[q]];
        seed[q] = ph_seed(tp[q]->id, cp[q]->name);
    }
    double *ps = malloc(sizeof(double) * 12 * (size_t)n_clones * np), *dt = malloc(sizeof(double) * np);
    int *m = malloc(sizeof(int) * np), *steps = malloc(sizeof(int) * np), *off = malloc(sizeof(int) * (np + 1));
    pgh_draw_pairs(np, tp, cp, n_clones, dt_myr, seed, threads, ps, m, steps, dt);
    off[0] = 0;
    for (int q = 0; q < np; q++) {   /* compact: clones of pair q follow those of q-1 */
        if (off[q] != q * n_clones) memmove(ps + 12 * (size_t)off[q], ps + 12 * (size_t)q * n_clones, sizeof(double) * 12 * m[q]);
        off[q + 1] = off[q] + m[q];
    }
    double *r50 = malloc(sizeof(double) * np), *rt = malloc(sizeof(double) * np);
    for (int q = 0; q < np; q++) { r50[q] = cp[q]->r50_pc; rt[q] = cp[q]->rtot_pc; }
    PhResult *res = malloc(sizeof(PhResult) * np);
    int rc = pgx_pair(ctx, np, off, ps, steps, dt, r50, rt, res, NULL);
    if (rc) {
        fprintf(stderr, "phygas_cli: pair batch: %s\n", pgx_last_error(ctx));
    } else {
        for (int q = 0; q < np; q++) {
            const PhResult *r = &res[q];
            printf("%s %s %c %d %.3f %.3f %.3f %.4f %.4f %.4f %.2f %.2f %.2f %.4f %.4f %.3f %.3f\n", tp[q]->id,
                   cp[q]->name, cp[q]->kind, r->n, r->d05, r->d50, r->d95, r->t05, r->t50, r->t95, r->v05, r->v50,
                   r->v95, r->f_r50, r->f_rtot, cp[q]->age16, cp[q]->age84);
        }
        fflush(stdout);
    }
    free(tp); free(cp); free(seed); free(ps); free(dt); free(m); free(steps); free(off); free(r50); free(rt); free(res);
    P->n = 0;
    return rc;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s clusters.txt targets.txt [n_clones] [dt_myr] [only=ID,...]\n", argv[0]);
        return 1;
    }
    int n_clones = argc > 3 ? atoi(argv[3]) : 1000;
    double dt = argc > 4 ? atof(argv[4]) : 0.05;
    const char *only = argc > 5 && strncmp(argv[5], "only=", 5) == 0 ? argv[5] + 5 : NULL;
    const char *be = getenv("PHYGAS_BATCH_CLONES");
    long batch = be && atol(be) > 0 ? atol(be) : (1L << 20);
    ph_init();
    PhCluster *cl;
    PhTarget *tg;
    int nc = ph_read_clusters(argv[1], &cl), nt = ph_read_targets(argv[2], &tg);
    if (nc <= 0 || nt <= 0) { fprintf(stderr, "can't read inputs (%d clusters, %d targets)\n", nc, nt); return 1; }
    if (n_clones > (1 << 26)) { fprintf(stderr, "phygas_cli: n_clones %d above 2^26\n", n_clones); return 1; }
    double tmax = 0;
    for (int i = 0; i < nc; i++) if (cl[i].tmax_myr > tmax) tmax = cl[i].tmax_myr;
    PgxContext *ctx;
    int rc = pgx_open(-1, &ctx);
    if (rc) { fprintf(stderr, "phygas_cli: no usable GPU (pgx_open: %d)\n", rc); return 1; }
    const int threads = pgh_default_threads();
    fprintf(stderr, "%d clusters (traced back up to %.0f Myr), %d targets, %d clones, dt %.3f Myr\n", nc, tmax, nt,
            n_clones, dt);
    long pairs = 0, done = 0;
    double t0 = now_s();
    /* the wanted targets, prefiltered against every cluster on the GPU in one call */
    int nw = 0, *widx = malloc(sizeof(int) * nt);
    PhTarget *wt = malloc(sizeof(PhTarget) * nt);
    for (int j = 0; j < nt; j++)
        if (wanted(tg[j].id, only)) { widx[nw] = j; wt[nw++] = tg[j]; }
    long cap = (long)nw * nc, np = 0;
    int *pti = malloc(sizeof(int) * (cap > 0 ? cap : 1)), *pci = malloc(sizeof(int) * (cap > 0 ? cap : 1));
    if (pgx_prefilter(ctx, wt, nw, cl, nc, threads, pti, pci, cap, &np)) {
        fprintf(stderr, "phygas_cli: prefilter: %s\n", pgx_last_error(ctx));
        return 1;
    }
    Pending P = {0, 0, NULL, NULL};
    for (long q = 0; q < np;) {
        const int w = pti[q];
        int kept = 0;
        for (; q < np && pti[q] == w; q++, kept++) {
            push(&P, widx[w], pci[q]);
            /* a batch holds about PHYGAS_BATCH_CLONES clones (at least one pair), whatever n_clones is */
            if ((long)P.n * (n_clones > 0 ? n_clones : 1) >= batch && flush(ctx, &P, tg, cl, n_clones, dt, threads))
                return 1;
        }
        pairs += kept;
        done++;
        fprintf(stderr, "%s: %d of %d clusters reachable (%.1f s so far)\n", tg[widx[w]].id, kept, nc, now_s() - t0);
    }
    done = nw;
    if (flush(ctx, &P, tg, cl, n_clones, dt, threads)) return 1;
    fprintf(stderr, "# done %ld targets, %ld pairs, %.1f s\n", done, pairs, now_s() - t0);
    pgx_close(ctx);
    return 0;
}
