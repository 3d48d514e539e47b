/* phygas_serve -- a seeded Poisson stream of jobs through libphygas_gb300's request loop (pgx_server_*): one JSON line
 * per job and a summary line with the p50/p99 job latency and the throughput.
 *
 *   phygas_serve clusters.txt stars.txt pulsars.txt [jobs=20] [rate_hz=1.0] [slots=3] [precision=mixed|fp64]
 *                [seed=1004] [plan]
 *
 * The stream: exponential inter-arrival times of mean 1/rate_hz; 40 % screen chunks and 20 % velocity-shuffled
 * control chunks of a window of stars.txt whose size is log-uniform in 1,000-20,000 stars (at most the file); 40 %
 * single-pulsar jobs, a line of pulsars.txt against every cluster that passes the prefilter, 1000 clones at dt
 * 0.05 Myr.  Screen chunks keep the rows with p_r50 >= 0.001, chi2_max 25.  Each job is submitted at its arrival
 * time; its latency is its end minus its arrival.  `plan` prints the stream and exits without touching a GPU.
 * PHYGAS_SERVE_HBM_GB sets the device-memory budget of the running jobs (default 80); PHYGAS_SERVE_MIX=pairs makes
 * every job a single-pulsar job (for the request loop's clone throughput under a backlog).
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "phygas_gb300.h"

static uint64_t sm_state;
static uint64_t sm_next(void) {                       /* splitmix64 */
    uint64_t z = (sm_state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double uni(void) { return (double)(sm_next() >> 11) * (1.0 / 9007199254740992.0); }

typedef struct {
    int kind, first, n;       /* targets [first, first + n) of the star or pulsar file */
    double arrive;
} Planned;

static const char *kind_name(int k) { return k == PGX_JOB_SCREEN ? "screen" : k == PGX_JOB_CONTROL ? "control" : "pulsar"; }

static int cmp_double(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

static double quantile(double *v, int n, double q) {      /* linear interpolation between order statistics */
    if (n <= 0) return 0.0;
    qsort(v, n, sizeof(double), cmp_double);
    double pos = q * (n - 1);
    int i = (int)pos;
    return i >= n - 1 ? v[n - 1] : v[i] + (pos - i) * (v[i + 1] - v[i]);
}

static void sleep_until(double t0, double t) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    double now = ts.tv_sec + ts.tv_nsec * 1e-9 - t0;
    if (t <= now) return;
    double d = t - now;
    struct timespec r = {(time_t)d, (long)((d - (time_t)d) * 1e9)};
    nanosleep(&r, NULL);
}

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s clusters.txt stars.txt pulsars.txt [jobs] [rate_hz] [slots] [mixed|fp64] [seed] "
                        "[plan]\n", argv[0]);
        return 1;
    }
    const int jobs = argc > 4 ? atoi(argv[4]) : 20;
    const double rate = argc > 5 ? atof(argv[5]) : 1.0;
    const int slots = argc > 6 ? atoi(argv[6]) : 3;
    const int precision = argc > 7 && !strcmp(argv[7], "fp64") ? PGX_FP64 : PGX_MIXED;
    sm_state = argc > 8 ? strtoull(argv[8], NULL, 10) : 1004;
    const int plan_only = argc > 9 && !strcmp(argv[9], "plan");
    if (jobs <= 0 || !(rate > 0) || slots <= 0) { fprintf(stderr, "phygas_serve: bad arguments\n"); return 1; }
    ph_init();
    PhCluster *cl;
    PhTarget *st, *pu;
    const int nc = ph_read_clusters(argv[1], &cl), ns = ph_read_targets(argv[2], &st), np = ph_read_targets(argv[3], &pu);
    if (nc <= 0 || ns <= 0 || np <= 0) { fprintf(stderr, "phygas_serve: can't read inputs\n"); return 1; }
    Planned *plan = malloc(sizeof(Planned) * jobs);
    const char *mix = getenv("PHYGAS_SERVE_MIX");
    const int pairs_only = mix && !strcmp(mix, "pairs");
    double t = 0;
    for (int i = 0; i < jobs; i++) {
        t += -log(1.0 - uni()) / rate;
        const double u = uni();
        Planned *p = &plan[i];
        p->arrive = t;
        if (pairs_only) {
            p->kind = PGX_JOB_PAIRS;
        } else if (u < 0.4 || u >= 0.6) {
            p->kind = u < 0.4 ? PGX_JOB_SCREEN : PGX_JOB_PAIRS;
        } else {
            p->kind = PGX_JOB_CONTROL;
        }
        if (p->kind == PGX_JOB_PAIRS) {
            p->n = 1;
            p->first = (int)(uni() * np) % np;
        } else {
            int n = (int)floor(1000.0 * pow(20.0, uni()));
            if (n > ns) n = ns;
            p->n = n;
            p->first = ns > n ? (int)(uni() * (ns - n + 1)) % (ns - n + 1) : 0;
        }
    }
    if (plan_only) {
        for (int i = 0; i < jobs; i++)
            printf("{\"job\": %d, \"kind\": \"%s\", \"first\": %d, \"n\": %d, \"arrive_s\": %.6f}\n", i,
                   kind_name(plan[i].kind), plan[i].first, plan[i].n, plan[i].arrive);
        return 0;
    }
    const char *hb = getenv("PHYGAS_SERVE_HBM_GB");
    PgxServer *srv;
    int rc = pgx_server_open(-1, slots, hb && atof(hb) > 0 ? atof(hb) : 80.0, cl, nc, 64, ph_screen_r, 0, &srv);
    if (rc) { fprintf(stderr, "phygas_serve: pgx_server_open: %d\n", rc); return 1; }
    long *id = malloc(sizeof(long) * jobs);
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    const double t0 = ts.tv_sec + ts.tv_nsec * 1e-9;
    PgxServerStats s0;
    pgx_server_stats(srv, &s0);                 /* the server clock at the start of the stream */
    for (int i = 0; i < jobs; i++) {
        sleep_until(t0, plan[i].arrive);
        PgxJob j;
        memset(&j, 0, sizeof j);
        j.kind = plan[i].kind;
        j.precision = precision;
        j.targets = j.kind == PGX_JOB_PAIRS ? pu + plan[i].first : st + plan[i].first;
        j.n_targets = plan[i].n;
        j.chi2_max = 25.0;
        j.p_min = 0.001;
        j.n_clones = 1000;
        j.dt_myr = 0.05;
        if ((rc = pgx_server_submit(srv, &j, &id[i]))) { fprintf(stderr, "phygas_serve: submit: %d\n", rc); return 1; }
    }
    double *lat = malloc(sizeof(double) * jobs), pairs = 0, clone_steps = 0, t_last = 0;
    int failed = 0;
    for (int i = 0; i < jobs; i++) {
        PgxJobResult r;
        pgx_server_wait(srv, id[i], &r);
        lat[i] = r.t_end - r.t_submit;
        if (r.status) failed++;
        if (r.kind == PGX_JOB_PAIRS) clone_steps += r.work; else pairs += r.work;
        if (r.t_end > t_last) t_last = r.t_end;
        printf("{\"job\": %d, \"kind\": \"%s\", \"n\": %d, \"status\": %d, \"slot\": %d, \"arrive_s\": %.4f, "
               "\"start_s\": %.4f, \"end_s\": %.4f, \"latency_s\": %.4f, \"n_out\": %ld, \"work\": %.6g, "
               "\"digest\": \"%016llx\"}\n", i, kind_name(r.kind), plan[i].n, r.status, r.slot, r.t_submit - s0.now_s,
               r.t_start - s0.now_s, r.t_end - s0.now_s, lat[i], r.n_out, r.work, (unsigned long long)r.digest);
        pgx_server_release(srv, id[i]);
    }
    PgxServerStats ss;
    pgx_server_stats(srv, &ss);
    const double wall = t_last - s0.now_s;
    double *l2 = malloc(sizeof(double) * jobs);
    memcpy(l2, lat, sizeof(double) * jobs);
    const double p50 = quantile(l2, jobs, 0.5), p99 = quantile(lat, jobs, 0.99);
    printf("{\"summary\": true, \"jobs\": %d, \"failed\": %d, \"rate_hz\": %g, \"slots\": %d, \"precision\": \"%s\", "
           "\"wall_s\": %.4f, \"latency_p50_s\": %.4f, \"latency_p99_s\": %.4f, \"screen_pairs_per_s\": %.6g, "
           "\"clone_steps_per_s\": %.6g, \"max_running\": %d, \"hbm_budget_gb\": %.1f, \"hbm_peak_gb\": %.2f}\n",
           jobs, failed, rate, slots, precision == PGX_FP64 ? "fp64" : "mixed", wall, p50, p99, pairs / wall,
           clone_steps / wall, ss.max_running, ss.hbm_budget_gb, ss.hbm_peak_gb);
    pgx_server_close(srv);
    return failed ? 1 : 0;
}
