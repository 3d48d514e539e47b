// pgx_serve.cu -- the serving loop of libphygas_gb300 (host code; no counterpart in the reference, whose BOINC app runs
// one work unit at a time).
//
// A server owns `slots` device contexts on one GPU.  Each context has its own stream and keeps the cluster table
// (orbits, covariances, the FP32 copies) and its work buffers resident between jobs.  Jobs -- screen chunks, control
// chunks, single-target pair jobs -- queue in arrival order.  A job starts when a slot is idle and the estimated
// device memory of the running jobs plus its own fits the budget (the first job of an empty GPU always starts).  Slot
// workers run their job's host part (draws, the prefilter's track starts) on their share of the host cores while
// other slots' kernels run, so jobs that arrive while others are on the GPU are admitted as slots and memory free up,
// and their work overlaps on the device.  A job's results depend only on its own inputs: every slot runs the same
// kernels on its own buffers, so a job gives the same bits alone and in a mix.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "phygas_gb300.h"
#include "../host/ph_host.h"

// persistent clone-kernel blocks per SM of a slot when several slots share the GPU
constexpr int kServeMcBlocksPerSm = 2;

namespace {

uint64_t fnv(uint64_t h, const void *p, size_t n) {
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ULL;
    return h;
}

struct HostBuf {
    void *p = nullptr;
    long cap = 0;
};

struct Job {
    long id = 0;
    PgxJob spec = {};
    std::vector<PhTarget> targets;
    size_t footprint = 0;
    bool done = false;
    PgxJobResult out = {};
    std::vector<PgxScreenRow> rows;
    std::vector<PhResult> res;
    std::vector<int> cluster;
};

}  // namespace

struct PgxServer {
    int device = 0, nslots = 0, host_threads = 1, n_samp = 64;
    size_t budget = 0, in_use = 0, peak = 0;
    double r_kernel = 2.0, tmax = 0.0;
    std::vector<PhCluster> clusters;
    std::vector<PgxContext *> ctx;
    std::vector<HostBuf> rows_buf;             // per slot: page-locked row buffer
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<long> queue;
    std::map<long, std::unique_ptr<Job>> jobs;
    long next_id = 1, submitted = 0, finished = 0;
    int running = 0, max_running = 0;
    int screens_running = 0;                   // screen and control jobs on the GPU (atomic access): while any runs,
                                               // the slots' clone kernels keep to kServeMcBlocksPerSm blocks per SM
    bool stop = false;
    std::vector<std::thread> workers;
    std::chrono::steady_clock::time_point t0;
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

// device memory a job needs while it runs, bytes: per screened star its 7 orbits (38.6 KB at 201 points), tracks
// (FP64 19.3 KB, FP32 9.6 KB), the per-pair filter state (17 B x clusters) and room for its kept pairs; per traced
// clone its start state, results and queue share (about 130 B); the 64 MiB allowance covers the prefilter's coarse
// tracks (24 B per point: 19.7 MB for 4,087 clusters of up to 201 points, kept by the slot)
size_t footprint(const PgxServer &s, const PgxJob &j) {
    const size_t nc = s.clusters.size();
    if (j.kind == PGX_JOB_PAIRS) return (size_t)j.n_targets * nc * (size_t)std::max(j.n_clones, 1) * 130 + (64u << 20);
    return (size_t)j.n_targets * (70000 + 40 * nc) + (64u << 20);
}

int run_screen(PgxServer &s, int slot, PgxContext *ctx, Job &job) {
    const PgxJob &j = job.spec;
    const int n = j.n_targets;
    std::vector<PhTarget> ctl;
    const PhTarget *t = job.targets.data();
    if (j.kind == PGX_JOB_CONTROL) {
        ctl.resize(n);
        pgh_control_targets(t, n, ctl.data());
        t = ctl.data();
    }
    std::vector<double> ps0((size_t)6 * n), sig((size_t)36 * n);
    std::vector<uint64_t> pre(n);
    pgh_draw_targets(t, n, s.n_samp, s.host_threads, ps0.data(), sig.data(), pre.data());
    // rows into the slot's page-locked buffer (grown when a chunk keeps more pairs than it holds)
    HostBuf &hb = s.rows_buf[slot];
    long nr = 0;
    int rc = pgx_screen_into(ctx, n, ps0.data(), sig.data(), pre.data(), s.tmax, j.chi2_max, j.precision,
                             (PgxScreenRow *)hb.p, hb.cap, &nr);
    if (rc == PGX_E_LIMIT) {
        pgx_host_free(hb.p);
        hb.cap = nr + nr / 4 + 4096;
        hb.p = pgx_host_alloc(sizeof(PgxScreenRow) * (size_t)hb.cap);
        if (!hb.p) { hb.cap = 0; return PGX_E_NOMEM; }
        rc = pgx_screen_fetch(ctx, (PgxScreenRow *)hb.p, nr);
    }
    if (rc) return rc;
    const PgxScreenRow *rows = (const PgxScreenRow *)hb.p;
    for (long h = 0; h < nr; h++)
        if (rows[h].p_r50 >= j.p_min) job.rows.push_back(rows[h]);
    job.out.n_out = (long)job.rows.size();
    job.out.work = (double)n * (double)s.clusters.size();
    job.out.digest = fnv(1469598103934665603ULL, job.rows.data(), job.rows.size() * sizeof(PgxScreenRow));
    return 0;
}

int run_pairs(PgxServer &s, PgxContext *ctx, Job &job) {
    const PgxJob &j = job.spec;
    const int nc = (int)s.clusters.size();
    std::vector<int> ti((size_t)j.n_targets * nc), ci((size_t)j.n_targets * nc);
    // the prefilter on the GPU: the slot's context keeps the cluster tracks, so each job traces only its targets
    long np = 0;
    const int prc = pgx_prefilter(ctx, job.targets.data(), j.n_targets, s.clusters.data(), nc, s.host_threads,
                                  ti.data(), ci.data(), (long)ti.size(), &np);
    if (prc) return prc;
    std::vector<int> ncl(np, j.n_clones);
    double work = 0;
    if (np > 0) {
        // the clone draws of each batch of pairs overlap the GPU's tracing of the one before (page-locked buffers)
        job.res.resize(np);
        const int rc = pgx_pair_targets(ctx, (int)np, job.targets.data(), ti.data(), s.clusters.data(), ci.data(),
                                        ncl.data(), j.dt_myr, s.host_threads, 0, job.res.data());
        if (rc) return rc;
        PgxStats st;
        pgx_stats(ctx, &st);
        work = (double)st.clone_steps;
    }
    job.cluster.assign(ci.begin(), ci.begin() + np);
    job.out.n_out = np;
    job.out.work = work;
    uint64_t h = fnv(1469598103934665603ULL, job.cluster.data(), job.cluster.size() * sizeof(int));
    job.out.digest = fnv(h, job.res.data(), job.res.size() * sizeof(PhResult));
    return 0;
}

// one slot: take the head of the queue when it fits the memory budget, run it, publish the result
void worker(PgxServer *s, int slot) {
    for (;;) {
        Job *job = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                if (s->queue.empty()) return s->stop;
                const Job &h = *s->jobs[s->queue.front()];
                return s->running == 0 || s->in_use + h.footprint <= s->budget;
            });
            if (s->queue.empty()) return;          // stopping, nothing left
            job = s->jobs[s->queue.front()].get();
            s->queue.pop_front();
            s->in_use += job->footprint;
            s->peak = std::max(s->peak, s->in_use);
            s->running++;
            s->max_running = std::max(s->max_running, s->running);
            job->out.t_start = s->now();
            job->out.slot = slot;
        }
        const bool screen = job->spec.kind != PGX_JOB_PAIRS;
        if (screen) __atomic_add_fetch(&s->screens_running, 1, __ATOMIC_ACQ_REL);
        const int rc = screen ? run_screen(*s, slot, s->ctx[slot], *job) : run_pairs(*s, s->ctx[slot], *job);
        if (screen) __atomic_sub_fetch(&s->screens_running, 1, __ATOMIC_ACQ_REL);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            job->out.status = rc;
            job->out.t_end = s->now();
            job->done = true;
            s->in_use -= job->footprint;
            s->running--;
            s->finished++;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

int pgx_server_open(int device, int slots, double hbm_budget_gb, const PhCluster *c, int nc, int n_samp,
                    double r_kernel, int host_threads, PgxServer **out) {
    if (!out || slots <= 0 || slots > 64 || !c || nc <= 0 || n_samp <= 0 || !(hbm_budget_gb > 0)) return PGX_E_ARG;
    *out = nullptr;
    std::unique_ptr<PgxServer> s(new PgxServer());
    s->nslots = slots;
    s->budget = (size_t)(hbm_budget_gb * 1e9);
    s->n_samp = n_samp;
    s->r_kernel = r_kernel;
    s->clusters.assign(c, c + nc);
    for (int i = 0; i < nc; i++) s->tmax = std::max(s->tmax, c[i].tmax_myr);
    const int cores = host_threads > 0 ? host_threads : pgh_default_threads();
    s->host_threads = std::max(1, cores / slots);
    // the cluster table: host draws once, the orbits on every slot's context
    std::vector<double> ps0((size_t)6 * nc), sig((size_t)36 * nc), tm(nc), r50(nc), rt(nc);
    std::vector<char> names((size_t)40 * nc, 0);
    pgh_draw_clusters(c, nc, n_samp, cores, ps0.data(), sig.data());
    for (int i = 0; i < nc; i++) {
        tm[i] = c[i].tmax_myr; r50[i] = c[i].r50_pc; rt[i] = c[i].rtot_pc;
        memcpy(&names[(size_t)40 * i], c[i].name, 40);
    }
    for (int k = 0; k < slots; k++) {
        PgxContext *ctx = nullptr;
        int rc = pgx_open(device, &ctx);
        if (rc) {
            for (PgxContext *x : s->ctx) pgx_close(x);
            return rc;
        }
        s->ctx.push_back(ctx);
        rc = pgx_screen_clusters(ctx, nc, ps0.data(), sig.data(), tm.data(), r50.data(), rt.data(), names.data(),
                                 r_kernel);
        // a pair job's persistent clone kernel would hold nearly every register of the GPU until its batch ends,
        // and the other slots' screens would wait for it: with more than one slot, a batch launched while a screen
        // or control job runs keeps to kServeMcBlocksPerSm blocks per SM, and one launched while none does takes the
        // whole GPU (pair jobs beside each other share it as concurrent kernels)
        if (rc == 0 && slots > 1) rc = pgx_pair_blocks_while(ctx, kServeMcBlocksPerSm, &s->screens_running);
        if (rc) {
            for (PgxContext *x : s->ctx) pgx_close(x);
            return rc;
        }
    }
    s->device = device;
    s->rows_buf.resize(slots);
    s->t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < slots; k++) s->workers.emplace_back(worker, s.get(), k);
    *out = s.release();
    return 0;
}

int pgx_server_submit(PgxServer *s, const PgxJob *job, long *id) {
    if (!s || !job || !id) return PGX_E_ARG;
    if (job->n_targets <= 0 || !job->targets) return PGX_E_ARG;
    if (job->kind != PGX_JOB_SCREEN && job->kind != PGX_JOB_CONTROL && job->kind != PGX_JOB_PAIRS) return PGX_E_ARG;
    if (job->kind == PGX_JOB_PAIRS && (job->n_clones < 0 || job->n_clones > (1 << 26) || !(job->dt_myr > 0)))
        return PGX_E_ARG;
    if (job->kind != PGX_JOB_PAIRS && job->precision != PGX_MIXED && job->precision != PGX_FP64) return PGX_E_ARG;
    std::unique_ptr<Job> j(new Job());
    j->spec = *job;
    j->targets.assign(job->targets, job->targets + job->n_targets);
    j->spec.targets = nullptr;
    j->footprint = footprint(*s, *job);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return PGX_E_ARG;
        j->id = s->next_id++;
        j->out.kind = job->kind;
        j->out.t_submit = s->now();
        j->out.status = -1;
        *id = j->id;
        s->queue.push_back(j->id);
        s->jobs[j->id] = std::move(j);
        s->submitted++;
    }
    s->cv_work.notify_all();
    return 0;
}

static Job *find(PgxServer *s, long id) {
    auto it = s->jobs.find(id);
    return it == s->jobs.end() ? nullptr : it->second.get();
}

int pgx_server_wait(PgxServer *s, long id, PgxJobResult *out) {
    if (!s) return PGX_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    Job *j = find(s, id);
    if (!j) return PGX_E_ARG;
    s->cv_done.wait(lk, [&] { return j->done; });
    if (out) *out = j->out;
    return 0;
}

int pgx_server_wait_for(PgxServer *s, long id, double timeout_s, PgxJobResult *out) {
    if (!s || !(timeout_s >= 0.0)) return PGX_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    Job *j = find(s, id);
    if (!j) return PGX_E_ARG;
    const bool done = s->cv_done.wait_for(lk, std::chrono::duration<double>(std::min(timeout_s, 1e7)),
                                          [&] { return j->done; });
    if (out) *out = j->out;
    return done ? 0 : PGX_E_TIMEOUT;
}

int pgx_server_query(PgxServer *s, long id, PgxJobResult *out) {
    if (!s) return PGX_E_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    Job *j = find(s, id);
    if (!j) return PGX_E_ARG;
    if (out) *out = j->out;
    return j->done ? 0 : PGX_E_PENDING;
}

long pgx_server_rows(PgxServer *s, long id, PgxScreenRow *rows, long cap) {
    if (!s) return -1;
    std::lock_guard<std::mutex> lk(s->mu);
    Job *j = find(s, id);
    if (!j || !j->done) return -1;
    const long n = (long)j->rows.size();
    if (rows) memcpy(rows, j->rows.data(), sizeof(PgxScreenRow) * (size_t)std::min(n, std::max(cap, 0L)));
    return n;
}

long pgx_server_pairs(PgxServer *s, long id, PhResult *res, int *cluster, long cap) {
    if (!s) return -1;
    std::lock_guard<std::mutex> lk(s->mu);
    Job *j = find(s, id);
    if (!j || !j->done) return -1;
    const long n = (long)j->res.size();
    const size_t k = (size_t)std::min(n, std::max(cap, 0L));
    if (res) memcpy(res, j->res.data(), sizeof(PhResult) * k);
    if (cluster) memcpy(cluster, j->cluster.data(), sizeof(int) * k);
    return n;
}

void pgx_server_release(PgxServer *s, long id) {
    if (!s) return;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it != s->jobs.end() && it->second->done) s->jobs.erase(it);
}

int pgx_server_stats(PgxServer *s, PgxServerStats *out) {
    if (!s || !out) return PGX_E_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    out->submitted = s->submitted;
    out->finished = s->finished;
    out->queued = (long)s->queue.size();
    out->running = s->running;
    out->max_running = s->max_running;
    out->slots = s->nslots;
    out->hbm_budget_gb = (double)s->budget / 1e9;
    out->hbm_in_use_gb = (double)s->in_use / 1e9;
    out->hbm_peak_gb = (double)s->peak / 1e9;
    out->now_s = s->now();
    return 0;
}

void pgx_server_close(PgxServer *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    for (auto &b : s->rows_buf) pgx_host_free(b.p);
    for (PgxContext *c : s->ctx) pgx_close(c);
    delete s;
}

}  // extern "C"
