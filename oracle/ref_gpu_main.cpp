/* ref_gpu_main.cpp -- the reference-GPU comparator (test and measurement infrastructure, never the product).
 *
 * Runs the reference's own GPU kernels (pg_lin_k, pg_chi2_k, pg_finish_k, pg_pair_k of src/phygas_kernel_body.h,
 * compiled from the reference's source for sm_103a into oracle/_ref/ref_kernels.ptx by `make -C oracle
 * ref-gpu-ptx`) the way the reference's BOINC app drives them, so that they can be timed on a GB300 beside this
 * build's kernels:
 *   screen mode  the app's gpu_screen (src/main_phygas_boinc.cpp:59-178): cluster tracks as structure of arrays,
 *                batches of PHYGAS_BATCH_STARS stars (default 1024) whose draws and covariances come from the host,
 *                pg_lin_k / pg_chi2_k / pg_finish_k launched in slices sized by the app's rule (each launch aimed at
 *                0.25 s, src/phygas_gpu.h:57-64), the kept pairs (chi2 < chi2_max) selected and seeded on the
 *                host between the chi2 and finish launches, rows with p_r50 >= p_min printed;
 *   pair mode    the app's gpu_pair (src/main_phygas_boinc.cpp:187-301): clones drawn on the host by ph_pair_draw
 *                for every pair the prefilter (or a clusters= list) selects, batches of PHYGAS_BATCH_CLONES (default
 *                262,144) traced by pg_pair_k in step slices, reduced on the host by ph_pair_reduce.
 * Each kernel launch is synchronous, as in the reference's CUDA backend (src/phygas_cuda.cu:47-77).  The host
 * functions are the oracle's (bit-identical to the reference's).  This program is our own code over the CUDA driver
 * API; it restates the app's loops, it does not copy them.
 *
 * usage: ref_gpu clusters in ptx [j0 j1]
 *   in: a work unit, line 1 "PHYGAS 1 screen <chi2_max> <n_samp> <r_kernel> <p_min>" or "PHYGAS 1 pair <n_clones>
 *       <dt_myr>", then one target per line (14 fields, optionally "clusters=NAME,...").  Targets [j0, j1).
 *   stdout: the rows, as the app writes them (no "# done" line).
 *   stderr: the app's summary line, then "ref_gpu_time total <s> host <s> lin <s> <n> chi2 <s> <n> finish <s> <n>
 *           pair <s> <n> pairs <count> clones <count> clone_steps <count>" (seconds of synchronous launches and
 *           their counts; host = everything else inside the loop: draws, copies, selection, reduction).
 */
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

extern "C" {
#include "phygas.h"
}

namespace {

double now_s() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + ts.tv_nsec * 1e-9;
}

void ck(CUresult r, const char *what) {
    if (r != CUDA_SUCCESS) {
        const char *s = nullptr;
        cuGetErrorString(r, &s);
        fprintf(stderr, "ref_gpu: %s: %s\n", what, s ? s : "?");
        exit(1);
    }
}

int env_int(const char *name, int def) {
    const char *v = getenv(name);
    const int x = v ? atoi(v) : 0;
    return x > 0 ? x : def;
}

// the app's launch-size rule: aim the next launch at 0.25 s, grow at most 4x, stay within [1, max_k]
int next_slice(int k, double elapsed, int max_k) {
    double want = elapsed > 1e-4 ? k * (0.25 / elapsed) : k * 4.0;
    want = std::min(want, k * 4.0);
    want = std::min(want, (double)max_k);
    return std::max(1, (int)want);
}

struct Dev {
    CUdeviceptr p = 0;
    size_t n = 0;
    void alloc(size_t bytes) { ck(cuMemAlloc(&p, bytes ? bytes : 8), "cuMemAlloc"); n = bytes; }
    void put(const void *h, size_t bytes) { if (bytes) ck(cuMemcpyHtoD(p, h, bytes), "cuMemcpyHtoD"); }
    void get(void *h, size_t bytes) const { if (bytes) ck(cuMemcpyDtoH(h, p, bytes), "cuMemcpyDtoH"); }
    void free_() { if (p) cuMemFree(p); p = 0; }
};

struct Timing {
    double s[4] = {0, 0, 0, 0};   // lin, chi2, finish, pair
    long n[4] = {0, 0, 0, 0};
};

struct Kernels {
    CUfunction lin, chi2, finish, pair;
};

// one synchronous launch of n threads in blocks of 128 (the backend's kThreads), timed
double launch(CUfunction f, int n, void **args, Timing &T, int which) {
    const double t0 = now_s();
    ck(cuLaunchKernel(f, (unsigned)((n + 127) / 128), 1, 1, 128, 1, 1, 0, nullptr, args, nullptr), "launch");
    ck(cuCtxSynchronize(), "kernel");
    const double dt = now_s() - t0;
    T.s[which] += dt;
    T.n[which]++;
    return dt;
}

const double kPrm[9] = {milkyway_potential_default.bulge_GM, milkyway_potential_default.bulge_b,
                        milkyway_potential_default.disk_GM,  milkyway_potential_default.disk_a,
                        milkyway_potential_default.disk_b,   milkyway_potential_default.halo_GM,
                        milkyway_potential_default.halo_a,   milkyway_potential_default.halo_cutoff,
                        milkyway_potential_default.halo_gamma};

int screen(const Kernels &K, const PhTarget *tg, int j0, int j1, const PhCluster *cl, int nc, const PhLin *clin,
           double tmax, double chi2_max, int n_samp, double p_min, Timing &T) {
    const int npts = (int)ceil(tmax / PH_PRE_STEP_MYR) + 1;
    std::vector<double> csoa((size_t)npts * 12 * nc, 0.0), R2s(nc), r50s(nc), rts(nc);
    std::vector<int> cn(nc);
    for (int ci = 0; ci < nc; ci++) {
        const PhLin &L = clin[ci];
        cn[ci] = L.n;
        for (int k = 0; k < L.n && k < npts; k++) {
            const double v[12] = {L.pos[k].x, L.pos[k].y, L.pos[k].z, L.vel[k].x, L.vel[k].y, L.vel[k].z,
                                  L.S[k][0], L.S[k][1], L.S[k][2], L.S[k][3], L.S[k][4], L.S[k][5]};
            for (int c = 0; c < 12; c++) csoa[((size_t)k * 12 + c) * nc + ci] = v[c];
        }
        const double R = (ph_screen_r > 0 ? ph_screen_r * cl[ci].r50_pc : cl[ci].rtot_pc) / 1000.0;
        R2s[ci] = R * R;
        r50s[ci] = cl[ci].r50_pc / 1000.0;
        rts[ci] = cl[ci].rtot_pc / 1000.0;
    }
    Dev d_csoa, d_cn, d_R2, d_r50, d_rt, d_prm;
    d_csoa.alloc(8 * csoa.size()); d_csoa.put(csoa.data(), 8 * csoa.size());
    d_cn.alloc(4 * (size_t)nc); d_cn.put(cn.data(), 4 * (size_t)nc);
    d_R2.alloc(8 * (size_t)nc); d_R2.put(R2s.data(), 8 * (size_t)nc);
    d_r50.alloc(8 * (size_t)nc); d_r50.put(r50s.data(), 8 * (size_t)nc);
    d_rt.alloc(8 * (size_t)nc); d_rt.put(rts.data(), 8 * (size_t)nc);
    d_prm.alloc(sizeof kPrm); d_prm.put(kPrm, sizeof kPrm);
    const int B = env_int("PHYGAS_BATCH_STARS", 1024);
    Dev ps0d, sigd, state, trk, chi2d, kbd, sbd;
    ps0d.alloc(8 * 6 * (size_t)B); sigd.alloc(8 * 36 * (size_t)B); state.alloc(8 * 63 * (size_t)B);
    trk.alloc(8 * 12 * (size_t)npts * B); chi2d.alloc(8 * (size_t)B * nc); kbd.alloc(4 * (size_t)B * nc);
    sbd.alloc(8 * (size_t)B * nc);
    fprintf(stderr, "GPU screening: %d stars per batch, %d clusters, %d points per track\n", B, nc, npts);
    const double dt = -PH_PRE_STEP_MYR / PH_LIN_SUB, eps_pos = PH_LIN_EPS_POS, eps_vel = PH_LIN_EPS_VEL;
    int sub = PH_LIN_SUB;
    std::vector<double> ps0(6 * (size_t)B), sig(36 * (size_t)B), chi2((size_t)B * nc), sb((size_t)B * nc);
    std::vector<int> kb((size_t)B * nc);
    int lin_slice = 4, chi2_slice = 65536, fin_slice = 16384;
    const double t_start = now_s();
    for (int b0 = j0; b0 < j1; b0 += B) {
        int nb = std::min(B, j1 - b0);
        for (int s = 0; s < nb; s++) {
            double S6[6][6];
            ph_lin_target_init(&tg[b0 + s], n_samp, ph_seed("lin", tg[b0 + s].id), &ps0[6 * s], S6);
            memcpy(&sig[36 * s], S6, sizeof S6);
        }
        ps0d.put(ps0.data(), 8 * 6 * (size_t)nb);
        sigd.put(sig.data(), 8 * 36 * (size_t)nb);
        for (int k = 0; k < npts;) {
            int nk = std::min(npts - k, lin_slice), k0 = k, np_ = npts, ns = nb;
            void *a[] = {&ps0d.p, &sigd.p, &state.p, &trk.p, &d_prm.p, (void *)&eps_pos, (void *)&eps_vel,
                         (void *)&dt, &sub, &k0, &nk, &np_, &ns};
            const double e = launch(K.lin, nb, a, T, 0);
            k += nk;
            lin_slice = next_slice(nk, e, npts);
        }
        const int total = nb * nc;
        for (int p = 0; p < total;) {
            int np = std::min(total - p, chi2_slice), p0 = p, nbb = nb, ncc = nc, npp = npts;
            void *a[] = {&trk.p, &d_csoa.p, &d_cn.p, &d_R2.p, &nbb, &ncc, &npp, &p0, &np, &chi2d.p, &kbd.p, &sbd.p};
            const double e = launch(K.chi2, np, a, T, 1);
            p += np;
            chi2_slice = next_slice(np, e, total);
        }
        chi2d.get(chi2.data(), 8 * (size_t)total);
        kbd.get(kb.data(), 4 * (size_t)total);
        sbd.get(sb.data(), 8 * (size_t)total);
        std::vector<int> hs, hc, hkb;
        std::vector<double> hsb, hchi2;
        std::vector<unsigned long long> hseed;
        for (int s = 0; s < nb; s++)
            for (int ci = 0; ci < nc; ci++) {
                const size_t i = (size_t)s * nc + ci;
                if (!(chi2[i] < chi2_max)) continue;
                hs.push_back(s); hc.push_back(ci); hkb.push_back(kb[i]); hsb.push_back(sb[i]);
                hchi2.push_back(chi2[i]);
                hseed.push_back(ph_seed(tg[b0 + s].id, cl[ci].name));
            }
        const int nh = (int)hs.size();
        std::vector<double> res(6 * (size_t)nh);
        if (nh > 0) {
            Dev b_hs, b_hc, b_hkb, b_hsb, b_seed, b_out;
            b_hs.alloc(4 * (size_t)nh); b_hs.put(hs.data(), 4 * (size_t)nh);
            b_hc.alloc(4 * (size_t)nh); b_hc.put(hc.data(), 4 * (size_t)nh);
            b_hkb.alloc(4 * (size_t)nh); b_hkb.put(hkb.data(), 4 * (size_t)nh);
            b_hsb.alloc(8 * (size_t)nh); b_hsb.put(hsb.data(), 8 * (size_t)nh);
            b_seed.alloc(8 * (size_t)nh); b_seed.put(hseed.data(), 8 * (size_t)nh);
            b_out.alloc(48 * (size_t)nh);
            for (int h = 0; h < nh;) {
                int n = std::min(nh - h, fin_slice), h0 = h, ncc = nc, npp = npts;
                void *a[] = {&trk.p, &d_csoa.p, &d_cn.p, &d_r50.p, &d_rt.p, &ncc, &npp, &b_hs.p, &b_hc.p, &b_hkb.p,
                             &b_hsb.p, &b_seed.p, &h0, &n, &b_out.p};
                const double e = launch(K.finish, n, a, T, 2);
                h += n;
                fin_slice = next_slice(n, e, nh);
            }
            b_out.get(res.data(), 48 * (size_t)nh);
            b_hs.free_(); b_hc.free_(); b_hkb.free_(); b_hsb.free_(); b_seed.free_(); b_out.free_();
        }
        for (int h = 0; h < nh; h++) {
            const double *r = &res[6 * (size_t)h];
            if (r[3] < p_min) continue;
            const PhCluster &c = cl[hc[h]];
            printf("%s %s %c %.3f %.3f %.2f %.2f %.4f %.4f %.2f\n", tg[b0 + hs[h]].id, c.name, c.kind, hchi2[h], r[0],
                   r[1], r[2], r[3], r[4], r[5]);
        }
        fflush(stdout);
    }
    fprintf(stderr, "GPU screening: %d stars in %.1f s\n", j1 - j0, now_s() - t_start);
    for (Dev *x : {&d_csoa, &d_cn, &d_R2, &d_r50, &d_rt, &d_prm, &ps0d, &sigd, &state, &trk, &chi2d, &kbd, &sbd})
        x->free_();
    return 0;
}

bool listed(const char *name, const char *list) {
    const size_t n = strlen(name);
    for (const char *p = list; (p = strstr(p, name)) != nullptr; p += n)
        if ((p == list || p[-1] == ',') && (p[n] == ',' || p[n] == '\0')) return true;
    return false;
}

int pairs(const Kernels &K, const PhTarget *tg, char *const *only, int j0, int j1, const PhCluster *cl, int nc,
          const PhTrack *ctr, double tmax, int n_clones, double dt_myr, Timing &T, long &n_pairs, long &n_cl,
          long long &clone_steps) {
    int batch = std::max(env_int("PHYGAS_BATCH_CLONES", 262144), n_clones);
    const int cap = 4 * batch;
    Dev d_prm, d_ps, d_steps, d_dts, d_st, d_res;
    d_prm.alloc(sizeof kPrm); d_prm.put(kPrm, sizeof kPrm);
    d_ps.alloc(8 * 12 * (size_t)cap); d_steps.alloc(4 * (size_t)cap); d_dts.alloc(8 * (size_t)cap);
    d_st.alloc(8 * 21 * (size_t)cap); d_res.alloc(8 * 3 * (size_t)cap);
    fprintf(stderr, "GPU pairs: %d clones per pair, up to %d clones per batch\n", n_clones, cap);
    struct Pend { int j, ci, m; size_t off; };
    struct Done { int j, ci; PhResult r; };
    std::vector<Pend> pend;
    std::vector<Done> done;
    std::vector<double> cps, cdts, res;
    std::vector<int> csteps;
    int slice = 20;
    const double t_start = now_s();
    auto flush = [&]() {
        const int n = (int)csteps.size();
        if (n > 0) {
            int smax = 0;
            for (int s : csteps) smax = std::max(smax, s);
            d_ps.put(cps.data(), 8 * 12 * (size_t)n);
            d_steps.put(csteps.data(), 4 * (size_t)n);
            d_dts.put(cdts.data(), 8 * (size_t)n);
            for (int s0 = 0; s0 < smax;) {
                int k = std::min(smax - s0, slice), s0v = s0, nn = n;
                void *a[] = {&d_ps.p, &d_steps.p, &d_dts.p, &d_st.p, &d_res.p, &d_prm.p, &s0v, &k, &nn};
                const double e = launch(K.pair, n, a, T, 3);
                s0 += k;
                slice = next_slice(k, e, smax);
            }
            res.resize(3 * (size_t)n);
            d_res.get(res.data(), 8 * 3 * (size_t)n);
        }
        std::vector<double> b, t, v;
        for (const Pend &p : pend) {
            b.resize(p.m > 0 ? p.m : 1); t.resize(b.size()); v.resize(b.size());
            for (int k = 0; k < p.m; k++) {
                const double *r = &res[3 * (p.off + k)];
                b[k] = r[0]; t[k] = r[1]; v[k] = r[2];
            }
            Done d;
            d.j = p.j; d.ci = p.ci;
            ph_pair_reduce(&cl[p.ci], p.m, b.data(), t.data(), v.data(), &d.r);
            done.push_back(d);
        }
        pend.clear(); cps.clear(); csteps.clear(); cdts.clear();
    };
    auto emit = [&](int upto) {
        size_t i = 0;
        for (; i < done.size() && done[i].j < upto; i++) {
            const Done &d = done[i];
            const PhResult &r = d.r;
            printf("%s %s %c %d %.3f %.3f %.3f %.4f %.4f %.4f %.2f %.2f %.2f %.4f %.4f\n", tg[d.j].id, cl[d.ci].name,
                   cl[d.ci].kind, r.n, r.d05, r.d50, r.d95, r.t05, r.t50, r.t95, r.v05, r.v50, r.v95, r.f_r50,
                   r.f_rtot);
        }
        done.erase(done.begin(), done.begin() + i);
        fflush(stdout);
    };
    std::vector<double> ps(12 * (size_t)std::max(n_clones, 1));
    for (int j = j0; j < j1; j++) {
        PhTrack tt;
        ph_track_target(&tg[j], tmax, 32, ph_seed("track", tg[j].id), &tt);
        for (int i = 0; i < nc; i++) {
            if (only[j] ? !listed(cl[i].name, only[j]) : !ph_prefilter(&tt, &ctr[i], &cl[i])) continue;
            if ((int)csteps.size() + n_clones > cap) {
                flush();
                emit(j);
            }
            int steps;
            double dt;
            const int m = ph_pair_draw(&tg[j], &cl[i], n_clones, dt_myr, ph_seed(tg[j].id, cl[i].name), ps.data(),
                                       &steps, &dt);
            pend.push_back({j, i, m, csteps.size()});
            cps.insert(cps.end(), ps.begin(), ps.begin() + 12 * (size_t)m);
            for (int k = 0; k < m; k++) { csteps.push_back(steps); cdts.push_back(dt); }
            n_pairs++;
            n_cl += m;
            clone_steps += (long long)m * steps;
        }
        ph_track_free(&tt);
        if ((int)csteps.size() >= batch || j + 1 == j1) {
            flush();
            emit(j + 1);
        }
    }
    fprintf(stderr, "GPU pairs: %d targets, %ld pairs, %ld clones in %.1f s\n", j1 - j0, n_pairs, n_cl,
            now_s() - t_start);
    for (Dev *x : {&d_prm, &d_ps, &d_steps, &d_dts, &d_st, &d_res}) x->free_();
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) { fprintf(stderr, "usage: ref_gpu clusters in ptx [j0 j1]\n"); return 2; }
    ph_init();
    PhCluster *cl;
    const int nc = ph_read_clusters(argv[1], &cl);
    FILE *f = fopen(argv[2], "r");
    if (nc <= 0 || !f) { fprintf(stderr, "can't read inputs\n"); return 1; }
    static char line[65536];
    char mode[16] = "";
    double p1 = 0, p2 = 0, p3 = 0, p4 = 0;
    if (!fgets(line, sizeof line, f) || sscanf(line, "PHYGAS 1 %15s %lf %lf %lf %lf", mode, &p1, &p2, &p3, &p4) < 3) {
        fprintf(stderr, "bad header\n");
        return 1;
    }
    std::vector<PhTarget> tg;
    std::vector<char *> only;
    while (fgets(line, sizeof line, f)) {
        PhTarget t = {};
        char srv[32], serv[32], kind[4];
        int used = 0;
        if (sscanf(line, "%39s %3s %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %31s %31s%n", t.id, kind, &t.ra, &t.dec,
                   &t.plx, &t.e_plx, &t.dist_pc, &t.e_lndist, &t.pmra, &t.e_pmra, &t.pmdec, &t.e_pmdec, srv, serv,
                   &used) != 14)
            continue;
        t.kind = kind[0];
        t.rv = strcmp(srv, "nan") ? atof(srv) : NAN;
        t.e_rv = strcmp(serv, "nan") ? atof(serv) : NAN;
        t.has_rv = !std::isnan(t.rv) && !std::isnan(t.e_rv);
        char *list = nullptr;
        const char *p = strstr(line + used, "clusters=");
        if (p) {
            const size_t len = strcspn(p + 9, " \r\n");
            if (len > 0) {
                list = (char *)malloc(len + 1);
                memcpy(list, p + 9, len);
                list[len] = 0;
            }
        }
        tg.push_back(t);
        only.push_back(list);
    }
    fclose(f);
    const int nt = (int)tg.size();
    int j0 = argc > 4 ? atoi(argv[4]) : 0, j1 = argc > 5 ? atoi(argv[5]) : nt;
    j1 = std::min(j1, nt);
    j0 = std::max(0, std::min(j0, j1));
    double tmax = 0;
    for (int i = 0; i < nc; i++) tmax = std::max(tmax, cl[i].tmax_myr);

    ck(cuInit(0), "cuInit");
    CUdevice dev;
    CUcontext ctx;
    ck(cuDeviceGet(&dev, 0), "cuDeviceGet");
    ck(cuDevicePrimaryCtxRetain(&ctx, dev), "cuDevicePrimaryCtxRetain");
    ck(cuCtxSetCurrent(ctx), "cuCtxSetCurrent");
    FILE *pf = fopen(argv[3], "rb");
    if (!pf) { fprintf(stderr, "ref_gpu: can't read %s\n", argv[3]); return 1; }
    std::string ptx;
    char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof buf, pf)) > 0) ptx.append(buf, got);
    fclose(pf);
    CUmodule mod;
    ck(cuModuleLoadData(&mod, ptx.c_str()), "cuModuleLoadData");
    Kernels K;
    ck(cuModuleGetFunction(&K.lin, mod, "pg_lin_k"), "pg_lin_k");
    ck(cuModuleGetFunction(&K.chi2, mod, "pg_chi2_k"), "pg_chi2_k");
    ck(cuModuleGetFunction(&K.finish, mod, "pg_finish_k"), "pg_finish_k");
    ck(cuModuleGetFunction(&K.pair, mod, "pg_pair_k"), "pg_pair_k");

    Timing T;
    long n_pairs = 0, n_cl = 0;
    long long clone_steps = 0;
    double t_prep = 0, t0 = now_s();
    if (!strcmp(mode, "screen")) {
        ph_screen_r = p3 > 0 ? p3 : 2.0;
        std::vector<PhLin> clin(nc);
        for (int i = 0; i < nc; i++) ph_lin_cluster(&cl[i], (int)p2, ph_seed("lin", cl[i].name), &clin[i]);
        t_prep = now_s() - t0;
        t0 = now_s();
        screen(K, tg.data(), j0, j1, cl, nc, clin.data(), tmax, p1, (int)p2, p4, T);
    } else if (!strcmp(mode, "pair")) {
        std::vector<PhTrack> ctr(nc);
        for (int i = 0; i < nc; i++) ph_track_cluster(&cl[i], 32, ph_seed("track", cl[i].name), &ctr[i]);
        t_prep = now_s() - t0;
        t0 = now_s();
        pairs(K, tg.data(), only.data(), j0, j1, cl, nc, ctr.data(), tmax, (int)p1, p2, T, n_pairs, n_cl,
              clone_steps);
    } else {
        fprintf(stderr, "unknown mode %s\n", mode);
        return 1;
    }
    const double total = now_s() - t0;
    const double kern = T.s[0] + T.s[1] + T.s[2] + T.s[3];
    fprintf(stderr, "ref_gpu_time prep %.6f total %.6f host %.6f lin %.6f %ld chi2 %.6f %ld finish %.6f %ld pair %.6f %ld "
                    "pairs %ld clones %ld clone_steps %lld\n",
            t_prep, total, total - kern, T.s[0], T.n[0], T.s[1], T.n[1], T.s[2], T.n[2], T.s[3], T.n[3], n_pairs,
            n_cl, clone_steps);
    cuModuleUnload(mod);
    cuDevicePrimaryCtxRelease(dev);
    return 0;
}
