// pgx_api.cu -- the C-ABI of libphygas_gb300 (include/phygas_gb300.h) and the GPU half of the drop-in API
// (include/phygas.h): device context, resident tables, work buffers, and the stage sequences.
//
// Stage sequence of one screen chunk (all on the context's stream, no host round trip before the kept-pair count):
//   k_stm_orbits -> k_stm_cov -> k_scan64 -> k_count_kept -> k_exclusive_scan -> [count to host] -> k_emit_kept
//   -> k_finish_prep -> k_finish64            (the FP64 path; the mixed path replaces scan..finish, pgx_mixed.cu)
// Pair Monte Carlo: one persistent k_pair_mc launch over a longest-first queue (+ k_pair_reduce_big).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstddef>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "phygas_gb300.h"
#include "pgx_kernels.h"
#include "pgx_mixed.h"
#include "pgx_prefilter.h"
#include "pgx_text.h"
#include "../host/ph_host.h"

static_assert(sizeof(pgx::PhResultDev) == sizeof(PhResult), "PhResult layout");
static_assert(offsetof(pgx::PhResultDev, d05) == offsetof(PhResult, d05), "PhResult layout");
static_assert(sizeof(pgx::ScreenRowDev) == sizeof(PgxScreenRow), "PgxScreenRow layout");

namespace {

struct Buf {
    void *p = nullptr;
    size_t cap = 0;
};

enum { EV_START, EV_ORBIT, EV_COV, EV_SCREEN, EV_SCAN, EV_SELECT, EV_FINISH, EV_PAIR0, EV_PAIR1, EV_N };

}  // namespace

// One staged chunk of stars: inputs (SoA), orbit scratch, the tracks the screen reads, the ids of the text lines,
// and the event that marks its tracks done
// Blocks per SM of a chunk's orbits traced beside another chunk's screen: few enough to leave the screen its
// registers (its FP32 and integer work and the orbits' FP64 work use different pipes), enough to finish first.
constexpr int kSideOrbitBlocksPerSm = 2;
// pgx_screen_stage splits chunks of at least this many stars in parts, so that exec can overlap one part's orbits
// with the previous part's screen.  A part's screen must outlast the next part's orbits, whose 2,000 KDK steps set a
// latency floor of a few ms whatever the part's size, so the first part, whose orbits are exposed, is small and the
// parts then grow: by default the first of about kPartPairs star-cluster pairs (2,447 stars at 4,087 clusters), each
// next 1.75 times the last (20,000 stars: 2,447, 4,282, 7,493 and 5,778).  Measured on 20,000 x 4,087: 87.9 ms a
// step, against 90.1, 88.5, 91.0 and 95.8 ms growing by 1.6, 1.7, 1.8 and 1.9, 89.0 by 1.5, 90.0 in 8 equal parts;
// beside the screens the orbits take 2 blocks per SM (1 block: 98.7 ms, 3: 89.8).  Earlier, before the block filter:
// 122 ms whole, 103 in 5 equal parts, 100 in 8, 104 in 12, 116 in 16.
constexpr int kSplitStars = 8192;
constexpr double kPartPairs = 1.0e7;

struct TrackSlot {
    int nt = 0, ns = 0;
    Buf ps0, sig21, prefix, opos, ovel, t64, t32, tlm, ids, blk;
    // the inputs the slot's tracks and screen read: its own buffers, or a part of a split chunk
    const double *in_ps0 = nullptr, *in_sig21 = nullptr;
    const uint64_t *in_prefix = nullptr;
    cudaEvent_t done = nullptr;
    char *h_stage = nullptr;                   // page-locked staging of the inputs (SoA), reused
    size_t h_stage_cap = 0;
};

struct PgxContext {
    int device = 0, sms = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[EV_N] = {};
    std::string err;
    // resident cluster table (original cluster order)
    int nc = 0, ncp = 0;
    Buf c64, c32, clm, cn, cR2, cr50, crt, cname, cblk;
    // the staged filter (PHYGAS_SCAN_TMA=1 at pgx_open): the cluster table cluster-major, and the wait flag
    bool scan_tma = false;
    Buf cblk_cm, c32_cm, clm_cm, werr;
    int nblk = 0, lm_pitch = 0;
    Buf x_draw, x_draw_ps;                     // device draws: records, seeds and outputs; clone slots
    // the mixed filter's block test (one test settles eight points of a pair); PHYGAS_SCAN_BLOCKS=0 at pgx_open
    // turns it off, and every point is walked (the same rows either way)
    bool scan_blocks = true;
    // device allocations made by ensure(), and the one that fails on purpose (PHYGAS_FAIL_ALLOC_AT; 0 = none)
    long allocs = 0, fail_alloc_at = 0;
    // the staged star chunks: two track slots, so that one chunk's orbits can run on the side stream while the
    // previous chunk is screened (pgx_screen_chunks); the single-chunk entry points use slot `cur`
    TrackSlot trk[2];
    int cur = 0;
    int split_min = kSplitStars;               // chunks of at least this many stars are split (0: never)
    int parts = 0;                             // in this many equal parts (0: parts ramping up from kPartPairs pairs)
    // a split chunk: pgx_screen_stage put part p's inputs (ps0[6][n], sig21[21][n], prefix[n]) at part_at[p] in
    // part_in; exec binds the parts to the two track slots in turn
    int nparts = 0;
    std::vector<int> part_n, part_off;
    std::vector<size_t> part_at;
    Buf part_in;
    char *h_part = nullptr;                    // page-locked staging of part_in
    size_t h_part_cap = 0;
    cudaStream_t side = nullptr;               // higher priority: the orbits' blocks start as soon as SMs free up
    // the screen's work buffers
    Buf chi2T, kbT, sbT, cnt, off, total, kept, fin, rows;
    // pgx_screen_chunks(_text): two chunks' rows or text on the device and in page-locked host memory, reused
    // across calls, and the labels of the text lines
    Buf rows_b[2];
    char *h_buf[2] = {};
    size_t h_cap[2] = {};
    Buf lab_names, lab_kinds, lab_age16, lab_age84;
    pgx::TextBufs text_bufs;
    pgx::PrefilterState pre;         // the prefilter's device tracks (the cluster side kept between calls)
    pgx::MixedBufs mixed;
    long n_rows = 0;
    // pair Monte Carlo
    Buf p_off, p_ps, p_steps, p_dt, p_r50, p_rt, p_items, p_q, p_done, p_cres, p_res, p_params;
    int mc_variant = 0;                        // launch shape of the clone kernel (pgx_tune_pair picks it)
    int mc_blocks_per_sm = 0;                  // > 0: the persistent clone kernels on at most this many blocks per SM
    const int *mc_busy = nullptr;              // set: the cap applies only while *mc_busy is nonzero at a launch
    double *h_clones[2] = {};                  // pgx_pair_targets: two batches of clones, page-locked, reused
    size_t h_clones_cap[2] = {};
    cudaGraphExec_t mc_exec[16] = {};          // prep + trace + reduce, captured once per shape, replayed
    cudaGraphExec_t mc_exec_capped[16] = {};   // the same with the grid capped (pgx_pair_blocks_while)
    // one-object helpers of the drop-in API
    Buf x_ps0, x_sig21, x_npts, x_opos, x_ovel, x_t64, x_t32, x_lm;
    PgxStats stats = {};
};

namespace {

int fail(PgxContext *c, int code, const char *fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    if (c) c->err = b;
    return code;
}

#define CK(call)                                                                                             \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess)                                                                               \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? PGX_E_NOMEM : PGX_E_CUDA, "%s: %s (%s:%d)", #call, \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                                         \
    } while (0)
#define CKL() CK(cudaGetLastError())
#define RET(x)                  \
    do {                        \
        int r_ = (x);           \
        if (r_) return r_;      \
    } while (0)
#define MRET(x)                                 \
    do {                                        \
        int r_ = (x);                           \
        if (r_) {                               \
            ctx->err = ctx->mixed.err;          \
            return r_;                          \
        }                                       \
    } while (0)

int ensure(PgxContext *ctx, Buf &b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return 0;
    if (b.p) CK(cudaFree(b.p));
    b.p = nullptr;
    b.cap = 0;
    const size_t want = bytes + bytes / 4;
    // fault injection on the host (PHYGAS_FAIL_ALLOC_AT=N at pgx_open): the context's N-th device allocation reports
    // that the device is out of memory, as a failed cudaMalloc would, without touching the device
    if (++ctx->allocs == ctx->fail_alloc_at)
        return fail(ctx, PGX_E_NOMEM, "device allocation %ld of %zu bytes: out of memory (injected)", ctx->allocs, want);
    CK(cudaMalloc(&b.p, want));
    b.cap = want;
    return 0;
}

template <class T> T *P(Buf &b) { return reinterpret_cast<T *>(b.p); }

int npts_of(double tmax) { return (int)std::ceil(tmax / PH_PRE_STEP_MYR) + 1; }

// ps0 [n][6] -> [6][n]; sig [n][36] -> the 21 upper-triangle entries [21][n]
// per-object ps0[6] and Sigma0[6][6] -> SoA p6[6][n] and the upper triangle s21[21][n] (slot order: order[slot])
void to_soa_into(int n, const double *ps0, const double *sig, double *p6, double *s21, const int *order = nullptr) {
    for (int slot = 0; slot < n; slot++) {
        const int i = order ? order[slot] : slot;
        for (int c = 0; c < 6; c++) p6[(size_t)c * n + slot] = ps0[(size_t)6 * i + c];
        int q = 0;
        for (int a = 0; a < 6; a++)
            for (int b = a; b < 6; b++) s21[(size_t)q++ * n + slot] = sig[(size_t)36 * i + 6 * a + b];
    }
}

void to_soa(int n, const double *ps0, const double *sig, std::vector<double> &p6, std::vector<double> &s21,
            const int *order = nullptr) {
    p6.resize((size_t)6 * n);
    s21.resize((size_t)21 * n);
    to_soa_into(n, ps0, sig, p6.data(), s21.data(), order);
}

// nominal + neighbour orbits of N objects (ps0 / sig21 device SoA, npts per slot or uniform) into t64 / t32
// orbit_blocks > 0: the orbits on at most that many blocks (grid-stride), to share the GPU with other work
int run_lin(PgxContext *ctx, cudaStream_t st, int N, const double *d_ps0, const double *d_sig21, const int *d_npts,
            int nmax, Buf &opos, Buf &ovel, double *t64, float4 *t32, float *lm, bool timed, int orbit_blocks = 0) {
    RET(ensure(ctx, opos, (size_t)nmax * 21 * N * sizeof(double)));
    RET(ensure(ctx, ovel, (size_t)nmax * 3 * N * sizeof(double)));
    int g = (int)((7L * N + 127) / 128);
    if (orbit_blocks > 0) g = std::min(g, orbit_blocks);
    pgx::k_stm_orbits<<<g, 128, 0, st>>>(N, d_ps0, d_npts, nmax, P<double>(opos), P<double>(ovel));
    CKL();
    if (timed) CK(cudaEventRecord(ctx->ev[EV_ORBIT], st));
    const size_t work = (size_t)N * nmax;
    pgx::k_stm_cov<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(N, nmax, d_npts, P<double>(opos),
                                                                     P<double>(ovel), d_sig21, t64, t32, lm);
    CKL();
    if (timed) CK(cudaEventRecord(ctx->ev[EV_COV], st));
    ctx->stats.kernels += 2;
    return 0;
}

pgx::ScreenTables tables(PgxContext *ctx, TrackSlot &k) {
    pgx::ScreenTables T;
    T.nt = k.nt; T.ns = k.ns; T.nc = ctx->nc; T.ncp = ctx->ncp; T.s_off = 0;
    T.t64 = P<double>(k.t64); T.t32 = P<float4>(k.t32); T.lm_t = P<float>(k.tlm);
    T.seed_prefix = k.in_prefix;
    T.c64 = P<double>(ctx->c64); T.c32 = P<float4>(ctx->c32); T.lm_c = P<float>(ctx->clm); T.cn = P<int>(ctx->cn);
    T.R2 = P<double>(ctx->cR2); T.r50 = P<double>(ctx->cr50); T.rtot = P<double>(ctx->crt);
    T.cname = P<char>(ctx->cname);
    if (ctx->scan_blocks && k.blk.p && ctx->cblk.p) {
        T.blk_t = P<float4>(k.blk);
        T.blk_c = P<float4>(ctx->cblk);
        if (ctx->scan_tma && ctx->cblk_cm.p) {
            T.blk_cm = P<float4>(ctx->cblk_cm);
            T.c32_cm = P<float4>(ctx->c32_cm);
            T.lm_cm = P<float>(ctx->clm_cm);
            T.nblk = ctx->nblk;
            T.lm_pitch = ctx->lm_pitch;
            T.wait_err = P<int>(ctx->werr);
        }
    }
    return T;
}

float elapsed(PgxContext *ctx, int a, int b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]) != cudaSuccess) return 0.f;
    return ms;
}

// Host inputs of nt stars (and, for text lines, their 40-byte ids) into track slot s, copied on stream st from the
// slot's page-locked staging area.
int stage_slot(PgxContext *ctx, int s, int nt, const double *ps0, const double *sig, const uint64_t *prefix,
               const char *ids, cudaStream_t st) {
    if (nt > (1 << 20)) return fail(ctx, PGX_E_LIMIT, "pgx_screen_stage: %d stars in one chunk (limit 2^20)", nt);
    TrackSlot &k = ctx->trk[s];
    const size_t b6 = (size_t)6 * nt * 8, b21 = (size_t)21 * nt * 8, bp = (size_t)nt * 8;
    const size_t bi = ids ? (size_t)40 * nt : 0;
    if (k.h_stage_cap < b6 + b21 + bp + bi) {
        pgx_host_free(k.h_stage);
        k.h_stage_cap = 0;
        const size_t cap = b6 + b21 + bp + (size_t)40 * nt;
        k.h_stage = (char *)pgx_host_alloc(cap);
        if (!k.h_stage) return fail(ctx, PGX_E_NOMEM, "pgx_screen_stage: %zu bytes of page-locked memory", cap);
        k.h_stage_cap = cap;
    }
    double *p6 = reinterpret_cast<double *>(k.h_stage), *s21 = p6 + (size_t)6 * nt;
    to_soa_into(nt, ps0, sig, p6, s21);
    memcpy(k.h_stage + b6 + b21, prefix, bp);
    if (ids) memcpy(k.h_stage + b6 + b21 + bp, ids, bi);
    RET(ensure(ctx, k.ps0, b6));
    RET(ensure(ctx, k.sig21, b21));
    RET(ensure(ctx, k.prefix, bp));
    CK(cudaMemcpyAsync(k.ps0.p, p6, b6, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(k.sig21.p, s21, b21, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(k.prefix.p, k.h_stage + b6 + b21, bp, cudaMemcpyHostToDevice, st));
    k.in_ps0 = P<double>(k.ps0);
    k.in_sig21 = P<double>(k.sig21);
    k.in_prefix = P<uint64_t>(k.prefix);
    if (ids) {
        RET(ensure(ctx, k.ids, bi));
        CK(cudaMemcpyAsync(k.ids.p, k.h_stage + b6 + b21 + bp, bi, cudaMemcpyHostToDevice, st));
    }
    CK(cudaStreamSynchronize(st));
    k.nt = nt;
    k.ns = 0;
    return 0;
}

// The orbits and covariances of slot s (nominal + 6 neighbours per star, S = A Sigma0 A^T) on stream st; the
// slot's event marks them done
int tracks_slot(PgxContext *ctx, int s, double tmax_myr, cudaStream_t st, bool timed, int orbit_blocks = 0) {
    TrackSlot &k = ctx->trk[s];
    const int ns = npts_of(tmax_myr), nt = k.nt;
    RET(ensure(ctx, k.t64, (size_t)ns * 12 * nt * 8));
    RET(ensure(ctx, k.t32, (size_t)ns * 3 * nt * 16));
    RET(ensure(ctx, k.tlm, (size_t)ns * nt * 4));
    RET(run_lin(ctx, st, nt, k.in_ps0, k.in_sig21, nullptr, ns, k.opos, k.ovel, P<double>(k.t64),
                P<float4>(k.t32), P<float>(k.tlm), timed, orbit_blocks));
    if (ctx->scan_blocks) {
        RET(ensure(ctx, k.blk, (size_t)((ns + pgx::kBlockPoints - 1) / pgx::kBlockPoints) * nt * 64));
        MRET(pgx::block_tables(st, nt, ns, nullptr, P<double>(k.t64), P<float>(k.tlm), nullptr, P<float4>(k.blk),
                               ctx->mixed.err));
        ctx->stats.kernels++;
    }
    CK(cudaEventRecord(k.done, st));
    k.ns = ns;
    return 0;
}

// part p of a split chunk into track slot s (its inputs in ctx->part_in)
void bind_part(PgxContext *ctx, int s, int p) {
    TrackSlot &k = ctx->trk[s];
    const int n = ctx->part_n[p];
    k.nt = n;
    k.ns = 0;
    k.in_ps0 = reinterpret_cast<const double *>(static_cast<const char *>(ctx->part_in.p) + ctx->part_at[p]);
    k.in_sig21 = k.in_ps0 + (size_t)6 * n;
    k.in_prefix = reinterpret_cast<const uint64_t *>(k.in_sig21 + (size_t)21 * n);
}

// ctx->rows with room for `rows` rows, the first `keep` of them kept
int rows_room(PgxContext *ctx, long keep, long rows) {
    const size_t need = (size_t)rows * sizeof(pgx::ScreenRowDev);
    if (ctx->rows.cap >= need) return 0;
    Buf old = ctx->rows;
    ctx->rows = Buf();
    RET(ensure(ctx, ctx->rows, need));
    if (keep > 0)
        CK(cudaMemcpyAsync(ctx->rows.p, old.p, (size_t)keep * sizeof(pgx::ScreenRowDev), cudaMemcpyDeviceToDevice,
                           ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (old.p) CK(cudaFree(old.p));
    return 0;
}

// The screen of slot s on the main stream, after its tracks (which may run on another stream): the scan, the
// selection of the kept pairs and their 512 draws; the rows stay on the device (ctx->rows, *n_rows of them from row
// row_off on, star indices star_off + the slot's).
// tracks_timed: the tracks ran on the main stream right before, timed by EV_START / EV_ORBIT / EV_COV.
int screen_slot(PgxContext *ctx, int s, double cut, int precision, long *n_rows, bool tracks_timed, long row_off = 0,
                int star_off = 0) {
    TrackSlot &k = ctx->trk[s];
    const int nt = k.nt, nc = ctx->nc, ns = k.ns;
    CK(cudaStreamWaitEvent(ctx->st, k.done, 0));
    if (!tracks_timed) {
        ctx->stats = PgxStats();
        for (int e : {EV_START, EV_ORBIT, EV_COV}) CK(cudaEventRecord(ctx->ev[e], ctx->st));
    }
    CK(cudaEventRecord(ctx->ev[EV_SCREEN], ctx->st));
    pgx::ScreenTables T = tables(ctx, k);
    T.s_off = star_off;
    int total = 0;
    if (precision == PGX_FP64) {
        const size_t pairs = (size_t)nt * nc;
        RET(ensure(ctx, ctx->chi2T, pairs * 8));
        RET(ensure(ctx, ctx->kbT, pairs * 4));
        RET(ensure(ctx, ctx->sbT, pairs * 8));
        RET(ensure(ctx, ctx->cnt, (size_t)nt * 4));
        RET(ensure(ctx, ctx->off, (size_t)nt * 4));
        RET(ensure(ctx, ctx->total, 16));
        dim3 g((nt + 127) / 128, std::min(nc, 65535));
        pgx::k_scan64<<<g, 128, 0, ctx->st>>>(T, cut, P<double>(ctx->chi2T), P<int>(ctx->kbT), P<double>(ctx->sbT));
        CKL();
        CK(cudaEventRecord(ctx->ev[EV_SCAN], ctx->st));
        pgx::k_count_kept<<<(nt + 127) / 128, 128, 0, ctx->st>>>(nt, nc, P<double>(ctx->chi2T), cut, P<int>(ctx->cnt));
        CKL();
        pgx::k_exclusive_scan<<<1, 1024, 0, ctx->st>>>(nt, P<int>(ctx->cnt), P<int>(ctx->off), P<int>(ctx->total));
        CKL();
        CK(cudaMemcpyAsync(&total, ctx->total.p, 4, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        RET(ensure(ctx, ctx->kept, (size_t)total * sizeof(pgx::KeptPair)));
        if (total > 0) {
            pgx::k_emit_kept<<<(nt + 127) / 128, 128, 0, ctx->st>>>(nt, nc, P<double>(ctx->chi2T), P<int>(ctx->kbT),
                                                                    P<double>(ctx->sbT), cut, P<int>(ctx->off),
                                                                    P<pgx::KeptPair>(ctx->kept));
            CKL();
        }
        CK(cudaEventRecord(ctx->ev[EV_SELECT], ctx->st));
        ctx->stats.kernels += 4;
    } else {
        MRET(pgx::mixed_select(ctx->st, T, cut, ctx->mixed, ctx->ev[EV_SCAN], &total, &ctx->stats));
        CK(cudaEventRecord(ctx->ev[EV_SELECT], ctx->st));
    }
    RET(ensure(ctx, ctx->fin, (size_t)total * sizeof(pgx::FinishIn)));
    RET(rows_room(ctx, row_off, row_off + total));
    pgx::ScreenRowDev *rows = P<pgx::ScreenRowDev>(ctx->rows) + row_off;
    if (total > 0) {
        const pgx::KeptPair *kp = precision == PGX_FP64 ? P<pgx::KeptPair>(ctx->kept) : pgx::mixed_kept(ctx->mixed);
        pgx::k_finish_prep<<<(total + 127) / 128, 128, 0, ctx->st>>>(T, total, kp, P<pgx::FinishIn>(ctx->fin),
                                                                     rows);
        CKL();
        if (precision == PGX_FP64) {
            pgx::k_finish64<<<(unsigned)(((size_t)total * 32 + 255) / 256), 256, 0, ctx->st>>>(
                total, P<pgx::FinishIn>(ctx->fin), rows);
            CKL();
        } else {
            MRET(pgx::mixed_finish(ctx->st, total, P<pgx::FinishIn>(ctx->fin), rows, ctx->mixed, &ctx->stats));
        }
        ctx->stats.kernels += 2;
    }
    CK(cudaEventRecord(ctx->ev[EV_FINISH], ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (T.wait_err) {
        int werr = 0;
        CK(cudaMemcpy(&werr, T.wait_err, 4, cudaMemcpyDeviceToHost));
        if (werr) return fail(ctx, PGX_E_CUDA, "screen: a bulk copy's wait in the filter ran out");
    }
    PgxStats &S = ctx->stats;
    S.ms_orbit = elapsed(ctx, EV_START, EV_ORBIT);
    S.ms_cov = elapsed(ctx, EV_ORBIT, EV_COV);
    S.ms_scan = elapsed(ctx, EV_SCREEN, EV_SCAN);
    S.ms_select = elapsed(ctx, EV_SCAN, EV_SELECT);
    S.ms_finish = elapsed(ctx, EV_SELECT, EV_FINISH);
    S.ms_total = elapsed(ctx, EV_START, EV_FINISH);
    S.pairs = (long)nt * nc;
    S.kept = total;
    S.body_steps = (long)nt * 7 * (ns - 1) * PH_LIN_SUB;
    S.orbit_body_steps = S.body_steps;
    ctx->n_rows = row_off + total;
    if (n_rows) *n_rows = total;
    return 0;
}


}  // namespace

// ---------------------------------------------------------------------------------------------------------------
extern "C" {

int pgx_open(int device, PgxContext **out) {
    PgxContext *ctx = nullptr;
    if (!out) return PGX_E_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return PGX_E_NODEV;
    if (device < 0) device = 0;
    if (device >= n) return PGX_E_ARG;
    ctx = new PgxContext();
    ctx->device = device;
    if (const char *e = getenv("PHYGAS_SCAN_BLOCKS")) ctx->scan_blocks = atoi(e) != 0;
    if (const char *e = getenv("PHYGAS_SCAN_TMA")) ctx->scan_tma = atoi(e) != 0;
    if (const char *e = getenv("PHYGAS_FAIL_ALLOC_AT")) ctx->fail_alloc_at = atol(e);
    int rc = 0;
    {
        auto init = [&]() -> int {
            CK(cudaSetDevice(device));
            CK(cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device));
            if (pgx::orbit_setup(device)) return fail(ctx, PGX_E_CUDA, "pgx_open: orbit force tables");
            CK(cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking));
            int lo = 0, hi = 0;
            CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            CK(cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, hi));
            for (auto &e : ctx->ev) CK(cudaEventCreate(&e));
            for (auto &k : ctx->trk) CK(cudaEventCreateWithFlags(&k.done, cudaEventDisableTiming));
            return 0;
        };
        rc = init();
    }
    if (rc) {
        pgx_close(ctx);
        return rc;
    }
    *out = ctx;
    return 0;
}

void pgx_close(PgxContext *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    Buf *bufs[] = {&ctx->c64, &ctx->c32, &ctx->clm, &ctx->x_lm, &ctx->cn, &ctx->cR2, &ctx->cr50, &ctx->crt,
                   &ctx->cname, &ctx->chi2T,
                   &ctx->kbT, &ctx->sbT, &ctx->cnt, &ctx->off, &ctx->total, &ctx->kept, &ctx->fin, &ctx->rows,
                   &ctx->p_off, &ctx->p_ps, &ctx->p_steps, &ctx->p_dt, &ctx->p_r50, &ctx->p_rt, &ctx->p_items,
                   &ctx->p_q, &ctx->p_done, &ctx->p_cres, &ctx->p_res, &ctx->p_params, &ctx->x_ps0, &ctx->x_sig21,
                   &ctx->x_npts,
                   &ctx->x_opos, &ctx->x_ovel, &ctx->x_t64, &ctx->x_t32, &ctx->rows_b[0], &ctx->rows_b[1],
                   &ctx->lab_names, &ctx->lab_kinds, &ctx->lab_age16, &ctx->lab_age84, &ctx->part_in,
                   &ctx->cblk, &ctx->x_draw, &ctx->x_draw_ps, &ctx->cblk_cm, &ctx->c32_cm, &ctx->clm_cm,
                   &ctx->werr};
    for (Buf *b : bufs)
        if (b->p) cudaFree(b->p);
    if (ctx->h_part) cudaFreeHost(ctx->h_part);
    for (auto &k : ctx->trk) {
        for (Buf *b : {&k.ps0, &k.sig21, &k.prefix, &k.opos, &k.ovel, &k.t64, &k.t32, &k.tlm, &k.ids, &k.blk})
            if (b->p) cudaFree(b->p);
        if (k.done) cudaEventDestroy(k.done);
        if (k.h_stage) cudaFreeHost(k.h_stage);
    }
    for (auto *h : ctx->h_buf)
        if (h) cudaFreeHost(h);
    for (auto *h : ctx->h_clones)
        if (h) cudaFreeHost(h);
    pgx::text_free(ctx->text_bufs);
    pgx::prefilter_free(ctx->pre);
    pgx::mixed_free(ctx->mixed);
    for (auto &g : ctx->mc_exec)
        if (g) cudaGraphExecDestroy(g);
    for (auto &g : ctx->mc_exec_capped)
        if (g) cudaGraphExecDestroy(g);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    delete ctx;
}

const char *pgx_last_error(const PgxContext *ctx) { return ctx ? ctx->err.c_str() : "no context"; }
void pgx_free(void *p) { free(p); }

uint64_t pgx_seed_prefix(const char *id) { return pgh_seed_prefix(id); }

int pgx_draw_targets(const PhTarget *t, int n, int n_samp, int threads, double *ps0, double *sig, uint64_t *prefix) {
    if (n < 0 || (n > 0 && (!t || !ps0 || !sig)) || n_samp < 0) return PGX_E_ARG;
    pgh_draw_targets(t, n, n_samp, threads > 0 ? threads : pgh_default_threads(), ps0, sig, prefix);
    return 0;
}

int pgx_draw_targets_gpu(PgxContext *ctx, const PhTarget *t, int n, int n_samp, double *ps0, double *sig,
                         uint64_t *prefix) {
    if (!ctx) return PGX_E_ARG;
    if (n < 0 || n_samp < 0 || (n > 0 && (!t || !ps0 || !sig))) return fail(ctx, PGX_E_ARG, "pgx_draw_targets_gpu");
    if (n == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    std::vector<uint64_t> seed(n);
    for (int i = 0; i < n; i++) {
        seed[i] = ph_seed("lin", t[i].id);
        if (prefix) prefix[i] = pgh_seed_prefix(t[i].id);
    }
    const size_t bt = (size_t)n * sizeof(PhTarget), bs = (size_t)n * 8, bo = (size_t)n * 42 * 8;
    RET(ensure(ctx, ctx->x_draw, bt + bs + bo + 64));
    char *b = P<char>(ctx->x_draw);
    PhTarget *dt = (PhTarget *)b;
    uint64_t *ds = (uint64_t *)(b + ((bt + 15) & ~(size_t)15));
    double *dp = (double *)(ds + n), *dg = dp + (size_t)6 * n;
    CK(cudaMemcpyAsync(dt, t, bt, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ds, seed.data(), bs, cudaMemcpyHostToDevice, ctx->st));
    ctx->stats = PgxStats();
    CK(cudaEventRecord(ctx->ev[EV_PAIR0], ctx->st));
    MRET(pgx::draw_targets_gpu(ctx->st, n, dt, n_samp, ds, dp, dg, ctx->mixed.err));
    CK(cudaEventRecord(ctx->ev[EV_PAIR1], ctx->st));
    CK(cudaMemcpyAsync(ps0, dp, (size_t)n * 6 * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(sig, dg, (size_t)n * 36 * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->stats.ms_total = elapsed(ctx, EV_PAIR0, EV_PAIR1);
    ctx->stats.kernels = 1;
    return 0;
}

int pgx_draw_pair_batch_gpu(PgxContext *ctx, int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c,
                            const int *ci, const int *n_clones, double dt_myr, int *clone_off, double *ps,
                            int *steps, double *dt, double *r50_pc, double *rtot_pc) {
    if (!ctx) return PGX_E_ARG;
    if (n_pairs < 0 || !clone_off || !(dt_myr > 0)) return fail(ctx, PGX_E_ARG, "pgx_draw_pair_batch_gpu");
    if (n_pairs > 0 && (!t || !ti || !c || !ci || !n_clones || !ps || !steps || !dt || !r50_pc || !rtot_pc))
        return fail(ctx, PGX_E_ARG, "pgx_draw_pair_batch_gpu");
    clone_off[0] = 0;
    if (n_pairs == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    // per pair on the host: seed, steps and dt as ph_pair_draw sets them, and a slot of n_clones clones
    int nt = 0, nc = 0;
    std::vector<uint64_t> seed(n_pairs);
    std::vector<long long> slot(n_pairs + 1, 0);
    for (int q = 0; q < n_pairs; q++) {
        if (ti[q] < 0 || ci[q] < 0 || n_clones[q] < 0 || n_clones[q] > pgx::kMaxPairClones)
            return fail(ctx, n_clones[q] > pgx::kMaxPairClones ? PGX_E_LIMIT : PGX_E_ARG,
                        "pgx_draw_pair_batch_gpu: pair %d", q);
        nt = std::max(nt, ti[q] + 1);
        nc = std::max(nc, ci[q] + 1);
        const PhCluster &cq = c[ci[q]];
        seed[q] = ph_seed(t[ti[q]].id, cq.name);
        steps[q] = (int)std::ceil(cq.tmax_myr / dt_myr);
        dt[q] = -cq.tmax_myr / steps[q];
        r50_pc[q] = cq.r50_pc;
        rtot_pc[q] = cq.rtot_pc;
        slot[q + 1] = slot[q] + n_clones[q];
    }
    const long long cap = slot[n_pairs];
    const size_t bt = ((size_t)nt * sizeof(PhTarget) + 15) & ~(size_t)15;
    const size_t bc = ((size_t)nc * sizeof(PhCluster) + 15) & ~(size_t)15;
    const size_t bi = (((size_t)n_pairs * 4 + 15) & ~(size_t)15);
    const size_t b8 = (size_t)n_pairs * 8;
    RET(ensure(ctx, ctx->x_draw, bt + bc + 4 * bi + 2 * b8 + 64));
    RET(ensure(ctx, ctx->x_draw_ps, (size_t)std::max(cap, 1LL) * 12 * 8 * 2));
    char *b = P<char>(ctx->x_draw);
    PhTarget *d_t = (PhTarget *)b;
    PhCluster *d_c = (PhCluster *)(b + bt);
    int *d_ti = (int *)(b + bt + bc), *d_ci = (int *)((char *)d_ti + bi), *d_n = (int *)((char *)d_ci + bi);
    int *d_m = (int *)((char *)d_n + bi);
    uint64_t *d_seed = (uint64_t *)((char *)d_m + bi);
    long long *d_slot = (long long *)(d_seed + n_pairs);
    double *d_ps = P<double>(ctx->x_draw_ps), *d_out = d_ps + (size_t)std::max(cap, 1LL) * 12;
    CK(cudaMemcpyAsync(d_t, t, (size_t)nt * sizeof(PhTarget), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_c, c, (size_t)nc * sizeof(PhCluster), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_ti, ti, (size_t)n_pairs * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_ci, ci, (size_t)n_pairs * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_n, n_clones, (size_t)n_pairs * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_seed, seed.data(), b8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d_slot, slot.data(), b8, cudaMemcpyHostToDevice, ctx->st));
    ctx->stats = PgxStats();
    CK(cudaEventRecord(ctx->ev[EV_PAIR0], ctx->st));
    MRET(pgx::draw_pairs_gpu(ctx->st, n_pairs, d_t, d_ti, d_c, d_ci, d_n, d_seed, d_slot, d_ps, d_m,
                             ctx->mixed.err));
    std::vector<int> m(n_pairs);
    CK(cudaMemcpyAsync(m.data(), d_m, (size_t)n_pairs * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    // the successful clones of pair q follow those of pair q - 1 (as ph_pair_draw leaves a pair's clones)
    long long off = 0;
    for (int q = 0; q < n_pairs; q++) {
        off += m[q];
        if (off > 2147483647LL) return fail(ctx, PGX_E_LIMIT, "pgx_draw_pair_batch_gpu: more than 2^31 clones");
        clone_off[q + 1] = (int)off;
    }
    CK(cudaMemcpyAsync(d_n, clone_off, (size_t)n_pairs * 4, cudaMemcpyHostToDevice, ctx->st));   // offsets
    MRET(pgx::compact_pairs_gpu(ctx->st, n_pairs, d_slot, d_n, d_m, d_ps, d_out, ctx->mixed.err));
    CK(cudaEventRecord(ctx->ev[EV_PAIR1], ctx->st));
    if (off > 0) CK(cudaMemcpyAsync(ps, d_out, (size_t)off * 12 * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->stats.ms_total = elapsed(ctx, EV_PAIR0, EV_PAIR1);
    ctx->stats.clones = off;
    ctx->stats.pairs = n_pairs;
    ctx->stats.kernels = 1;
    return 0;
}

int pgx_draw_clusters(const PhCluster *c, int n, int n_samp, int threads, double *ps0, double *sig) {
    if (n < 0 || (n > 0 && (!c || !ps0 || !sig)) || n_samp < 0) return PGX_E_ARG;
    pgh_draw_clusters(c, n, n_samp, threads > 0 ? threads : pgh_default_threads(), ps0, sig);
    return 0;
}

int pgx_control_targets(const PhTarget *t, int n, PhTarget *out) {
    if (n < 0 || (n > 0 && (!t || !out)) || (n > 0 && t == out)) return PGX_E_ARG;
    pgh_control_targets(t, n, out);
    return 0;
}

int pgx_prefilter_pairs(const PhTarget *t, int nt, const PhCluster *c, int nc, int threads, int *ti, int *ci,
                        long cap, long *n) {
    if (nt < 0 || nc < 0 || cap < 0 || !n || (nt > 0 && !t) || (nc > 0 && !c) || (cap > 0 && (!ti || !ci)))
        return PGX_E_ARG;
    const long r = pgh_prefilter_pairs(t, nt, c, nc, threads > 0 ? threads : pgh_default_threads(), ti, ci, cap);
    if (r < 0) return PGX_E_NOMEM;
    *n = r;
    return 0;
}

int pgx_draw_pair_batch(int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c, const int *ci,
                        const int *n_clones, double dt_myr, int threads, int *clone_off, double *ps, int *steps,
                        double *dt, double *r50_pc, double *rtot_pc) {
    if (n_pairs < 0 || !clone_off) return PGX_E_ARG;
    if (n_pairs > 0 && (!t || !ti || !c || !ci || !n_clones || !ps || !steps || !dt || !r50_pc || !rtot_pc))
        return PGX_E_ARG;
    for (int q = 0; q < n_pairs; q++)
        if (n_clones[q] < 0 || n_clones[q] > pgx::kMaxPairClones) return PGX_E_LIMIT;
    const int r = pgh_draw_pair_batch(n_pairs, t, ti, c, ci, n_clones, dt_myr,
                                      threads > 0 ? threads : pgh_default_threads(), clone_off, ps, steps, dt,
                                      r50_pc, rtot_pc);
    return r == 0 ? 0 : (r == -1 ? PGX_E_NOMEM : PGX_E_LIMIT);
}

int pgx_prefilter(PgxContext *ctx, const PhTarget *t, int nt, const PhCluster *c, int nc, int threads, int *ti,
                  int *ci, long cap, long *n) {
    if (!ctx) return PGX_E_ARG;
    if (nt < 0 || nc < 0 || cap < 0 || !n || (nt > 0 && !t) || (nc > 0 && !c) || (cap > 0 && (!ti || !ci)))
        return fail(ctx, PGX_E_ARG, "pgx_prefilter: bad args");
    CK(cudaSetDevice(ctx->device));
    pgx::PrefilterCounts cnt;
    std::string err;
    ctx->stats = PgxStats();
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = pgx::prefilter_pairs(ctx->st, ctx->pre, t, nt, c, nc, threads > 0 ? threads : pgh_default_threads(),
                                        ti, ci, cap, n, cnt, err);
    if (rc) return fail(ctx, rc, "pgx_prefilter: %s", err.c_str());
    ctx->stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    ctx->stats.ms_prefilter = cnt.ms_device;
    ctx->stats.prefilter_pairs = cnt.pairs;
    ctx->stats.prefilter_rechecked = cnt.rechecked;
    ctx->stats.body_steps = cnt.body_steps;
    ctx->stats.kernels = cnt.kernels;
    return 0;
}

int pgx_cluster_list(const PhCluster *c, int nc, const char *list, int *ci, int cap) {
    if (nc < 0 || (nc > 0 && !c) || cap < 0 || (cap > 0 && !ci)) return -PGX_E_ARG;
    if (!list) return 0;
    int m = 0;
    for (int i = 0; i < nc; i++) {
        // whole items of the list: the name bounded by the list's start or a comma, and by a comma or the end
        char name[sizeof c[i].name + 1];
        const size_t len = strnlen(c[i].name, sizeof c[i].name);
        if (len == 0) continue;
        memcpy(name, c[i].name, len);
        name[len] = '\0';
        bool hit = false;
        for (const char *p = list; !hit && (p = strstr(p, name)) != nullptr; p += len)
            hit = (p == list || p[-1] == ',') && (p[len] == ',' || p[len] == '\0');
        if (!hit) continue;
        if (m < cap) ci[m] = i;
        m++;
    }
    return m;
}

int pgx_pairs_with_lists(PgxContext *ctx, const PhTarget *t, int nt, const char *const *lists, const PhCluster *c,
                         int nc, int threads, int *ti, int *ci, long cap, long *n) {
    if (!ctx) return PGX_E_ARG;
    if (nt < 0 || nc < 0 || cap < 0 || !n || (nt > 0 && !t) || (nc > 0 && !c) || (cap > 0 && (!ti || !ci)))
        return fail(ctx, PGX_E_ARG, "pgx_pairs_with_lists: bad args");
    *n = 0;
    // the targets without a list through the GPU prefilter, in one call
    std::vector<int> pre_idx;
    std::vector<PhTarget> pre_t;
    for (int j = 0; j < nt; j++)
        if (!lists || !lists[j] || !lists[j][0]) {
            pre_idx.push_back(j);
            pre_t.push_back(t[j]);
        }
    const long pcap = (long)pre_t.size() * nc;
    std::vector<int> pti(std::max(pcap, 1L)), pci(std::max(pcap, 1L));
    long np = 0;
    if (!pre_t.empty()) RET(pgx_prefilter(ctx, pre_t.data(), (int)pre_t.size(), c, nc, threads, pti.data(), pci.data(),
                                          pcap, &np));
    // merge in target order: a listed target's clusters from its list, the others' from the prefilter
    std::vector<int> li(std::max(nc, 1));
    long m = 0, q = 0;
    size_t w = 0;
    for (int j = 0; j < nt; j++) {
        if (w < pre_idx.size() && pre_idx[w] == j) {
            for (; q < np && pti[q] == (int)w; q++, m++)
                if (m < cap) { ti[m] = j; ci[m] = pci[q]; }
            w++;
            continue;
        }
        const int k = pgx_cluster_list(c, nc, lists[j], li.data(), nc);
        for (int a = 0; a < k; a++, m++)
            if (m < cap) { ti[m] = j; ci[m] = li[a]; }
    }
    *n = m;
    return 0;
}

int pgx_prefilter_margin(PgxContext *ctx, double margin_kpc) {
    if (!ctx) return PGX_E_ARG;
    if (!(margin_kpc >= 0.0 && margin_kpc <= 1e6)) return fail(ctx, PGX_E_ARG, "pgx_prefilter_margin: %g", margin_kpc);
    ctx->pre.margin = margin_kpc;
    return 0;
}

int pgx_tracks(PgxContext *ctx, int n, const double *ps, const int *npts, double *pos) {
    if (!ctx) return PGX_E_ARG;
    if (n < 0 || (n > 0 && (!ps || !npts || !pos))) return fail(ctx, PGX_E_ARG, "pgx_tracks: bad args");
    for (int i = 0; i < n; i++)
        if (npts[i] < 1 || npts[i] > 200001) return fail(ctx, PGX_E_ARG, "pgx_tracks: npts[%d] = %d", i, npts[i]);
    CK(cudaSetDevice(ctx->device));
    std::string err;
    const int rc = pgx::coarse_tracks(ctx->st, ctx->pre, n, ps, npts, pos, err);
    if (rc) return fail(ctx, rc, "pgx_tracks: %s", err.c_str());
    return 0;
}

int pgx_stats(const PgxContext *ctx, PgxStats *out) {
    if (!ctx || !out) return PGX_E_ARG;
    *out = ctx->stats;
    return 0;
}

int pgx_peaks(PgxContext *ctx, double *fp64, double *fp32) {
    if (!ctx || !fp64 || !fp32) return PGX_E_ARG;
    CK(cudaSetDevice(ctx->device));
    const int blocks = ctx->sms * 8, threads = 256;
    RET(ensure(ctx, ctx->x_opos, (size_t)blocks * threads * 8));
    const int it64 = 2000, it32 = 32000;
    for (int rep = 0; rep < 2; rep++) {      // the first round warms up
        CK(cudaEventRecord(ctx->ev[EV_PAIR0], ctx->st));
        pgx::k_peak_dfma<<<blocks, threads, 0, ctx->st>>>(P<double>(ctx->x_opos), it64, 1.0000001, 1e-9);
        CKL();
        CK(cudaEventRecord(ctx->ev[EV_PAIR1], ctx->st));
        pgx::k_peak_ffma<<<blocks, threads, 0, ctx->st>>>(P<float>(ctx->x_opos), it32, 1.0000001f, 1e-9f);
        CKL();
        CK(cudaEventRecord(ctx->ev[EV_START], ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    const double n = (double)blocks * threads * 8 * 2;
    *fp64 = n * it64 / (elapsed(ctx, EV_PAIR0, EV_PAIR1) * 1e-3);
    *fp32 = n * it32 / (elapsed(ctx, EV_PAIR1, EV_START) * 1e-3);
    return 0;
}

int pgx_check_bounds(PgxContext *ctx, int n, const double *pos, const double *S, const double *R2, double cut,
                     double *v64, float *lb, float *ub, int *rej) {
    if (!ctx) return PGX_E_ARG;
    if (n <= 0 || !pos || !S || !R2 || !v64 || !lb || !ub || !rej) return fail(ctx, PGX_E_ARG, "pgx_check_bounds");
    CK(cudaSetDevice(ctx->device));
    const size_t in = (size_t)n * (12 + 12 + 1) * 8, out = (size_t)n * (8 + 4 + 4 + 4);
    RET(ensure(ctx, ctx->x_opos, in + out + 64));
    char *b = P<char>(ctx->x_opos);
    double *dp = (double *)b, *dS = dp + (size_t)12 * n, *dR = dS + (size_t)12 * n, *dv = dR + n;
    float *dl = (float *)(dv + n), *du = dl + n;
    int *dj = (int *)(du + n);
    CK(cudaMemcpyAsync(dp, pos, (size_t)12 * n * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(dS, S, (size_t)12 * n * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(dR, R2, (size_t)n * 8, cudaMemcpyHostToDevice, ctx->st));
    MRET(pgx::mixed_check_bounds(ctx->st, n, dp, dS, dR, cut, dv, dl, du, dj, ctx->mixed.err));
    CK(cudaMemcpyAsync(v64, dv, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(lb, dl, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(ub, du, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(rej, dj, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pgx_check_blocks(PgxContext *ctx, double tmax_myr, double chi2_max, long *counts) {
    if (!ctx) return PGX_E_ARG;
    if (!counts || !(chi2_max > 0) || !(tmax_myr > 0)) return fail(ctx, PGX_E_ARG, "pgx_check_blocks: bad args");
    if (ctx->nc <= 0 || ctx->nparts != 0 || ctx->trk[ctx->cur].nt <= 0)
        return fail(ctx, PGX_E_ARG, "pgx_check_blocks: stage one unsplit chunk against a cluster table first");
    if (!ctx->scan_blocks) return fail(ctx, PGX_E_ARG, "pgx_check_blocks: the block test is off (PHYGAS_SCAN_BLOCKS)");
    CK(cudaSetDevice(ctx->device));
    RET(tracks_slot(ctx, ctx->cur, tmax_myr, ctx->st, false));
    RET(ensure(ctx, ctx->total, sizeof(unsigned long long) * pgx::kCheckBlockCounts));
    const pgx::ScreenTables T = tables(ctx, ctx->trk[ctx->cur]);
    MRET(pgx::mixed_check_blocks(ctx->st, T, chi2_max, P<unsigned long long>(ctx->total), ctx->mixed.err));
    unsigned long long h[pgx::kCheckBlockCounts];
    CK(cudaMemcpyAsync(h, ctx->total.p, sizeof h, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int i = 0; i < pgx::kCheckBlockCounts; i++) counts[i] = (long)h[i];
    return 0;
}

int pgx_check_draws(PgxContext *ctx, int n, const double *fin11, const uint64_t *seed, double *ratio) {
    if (!ctx) return PGX_E_ARG;
    if (n <= 0 || !fin11 || !seed || !ratio) return fail(ctx, PGX_E_ARG, "pgx_check_draws");
    CK(cudaSetDevice(ctx->device));
    std::vector<pgx::FinishIn> h(n);
    for (int i = 0; i < n; i++) {
        const double *v = fin11 + (size_t)11 * i;
        pgx::FinishIn &f = h[i];
        f.mx = v[0]; f.my = v[1]; f.mz = v[2]; f.l00 = v[3]; f.l10 = v[4]; f.l20 = v[5];
        f.l11 = v[6]; f.l21 = v[7]; f.l22 = v[8]; f.r50 = v[9]; f.rt = v[10]; f.seed = seed[i];
    }
    RET(ensure(ctx, ctx->x_opos, (size_t)n * (sizeof(pgx::FinishIn) + 8) + 64));
    pgx::FinishIn *df = P<pgx::FinishIn>(ctx->x_opos);
    double *dr = reinterpret_cast<double *>(df + n);
    CK(cudaMemcpyAsync(df, h.data(), (size_t)n * sizeof(pgx::FinishIn), cudaMemcpyHostToDevice, ctx->st));
    MRET(pgx::mixed_check_draws(ctx->st, n, df, dr, ctx->mixed.err));
    CK(cudaMemcpyAsync(ratio, dr, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pgx_lin(PgxContext *ctx, int n, const double *ps0, const double *sig, const int *npts, double *pos, double *vel,
            double *S) {
    if (!ctx) return PGX_E_ARG;
    if (n < 0 || (n > 0 && (!ps0 || !sig || !npts || !pos || !vel || !S))) return fail(ctx, PGX_E_ARG, "pgx_lin: bad args");
    if (n == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    int nmax = 0;
    for (int i = 0; i < n; i++) {
        if (npts[i] < 1) return fail(ctx, PGX_E_ARG, "pgx_lin: npts[%d] = %d", i, npts[i]);
        nmax = std::max(nmax, npts[i]);
    }
    std::vector<double> p6, s21;
    to_soa(n, ps0, sig, p6, s21);
    RET(ensure(ctx, ctx->x_ps0, p6.size() * 8));
    RET(ensure(ctx, ctx->x_sig21, s21.size() * 8));
    RET(ensure(ctx, ctx->x_npts, (size_t)n * 4));
    RET(ensure(ctx, ctx->x_t64, (size_t)nmax * 12 * n * 8));
    RET(ensure(ctx, ctx->x_t32, (size_t)nmax * 3 * n * 16));
    RET(ensure(ctx, ctx->x_lm, (size_t)nmax * n * 4));
    CK(cudaMemcpyAsync(ctx->x_ps0.p, p6.data(), p6.size() * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->x_sig21.p, s21.data(), s21.size() * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->x_npts.p, npts, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->st));
    ctx->stats = PgxStats();
    RET(run_lin(ctx, ctx->st, n, P<double>(ctx->x_ps0), P<double>(ctx->x_sig21), P<int>(ctx->x_npts), nmax,
                ctx->x_opos, ctx->x_ovel, P<double>(ctx->x_t64), P<float4>(ctx->x_t32), P<float>(ctx->x_lm), false));
    std::vector<double> t((size_t)nmax * 12 * n);
    CK(cudaMemcpyAsync(t.data(), ctx->x_t64.p, t.size() * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    size_t o = 0;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < npts[i]; k++, o++) {
            const double *T = t.data() + (size_t)k * 12 * n + i;
            for (int c = 0; c < 3; c++) pos[3 * o + c] = T[(size_t)c * n];
            for (int c = 0; c < 3; c++) vel[3 * o + c] = T[(size_t)(3 + c) * n];
            for (int c = 0; c < 6; c++) S[6 * o + c] = T[(size_t)(6 + c) * n];
        }
    return 0;
}

int pgx_screen_clusters(PgxContext *ctx, int nc, const double *ps0, const double *sig, const double *tmax_myr,
                        const double *r50_pc, const double *rtot_pc, const char *names, double r_kernel) {
    if (!ctx) return PGX_E_ARG;
    if (nc <= 0 || !ps0 || !sig || !tmax_myr || !r50_pc || !rtot_pc || !names)
        return fail(ctx, PGX_E_ARG, "pgx_screen_clusters: bad args");
    CK(cudaSetDevice(ctx->device));
    std::vector<int> npts(nc), order(nc), col(nc);
    int nmax = 0;
    for (int i = 0; i < nc; i++) {
        npts[i] = npts_of(tmax_myr[i]);
        if (npts[i] < 1) return fail(ctx, PGX_E_ARG, "pgx_screen_clusters: tmax %g", tmax_myr[i]);
        nmax = std::max(nmax, npts[i]);
        order[i] = i;
    }
    // integrate longest first, so the lanes of a warp carry tracks of similar length
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return npts[a] > npts[b]; });
    std::vector<int> npts_slot(nc);
    for (int s = 0; s < nc; s++) npts_slot[s] = npts[order[s]];
    std::vector<double> p6, s21;
    to_soa(nc, ps0, sig, p6, s21, order.data());
    RET(ensure(ctx, ctx->x_ps0, p6.size() * 8));
    RET(ensure(ctx, ctx->x_sig21, s21.size() * 8));
    RET(ensure(ctx, ctx->x_npts, (size_t)nc * 4));
    RET(ensure(ctx, ctx->x_t64, (size_t)nmax * 12 * nc * 8));
    RET(ensure(ctx, ctx->x_t32, (size_t)nmax * 3 * nc * 16));
    RET(ensure(ctx, ctx->x_lm, (size_t)nmax * nc * 4));
    RET(ensure(ctx, ctx->c64, (size_t)nmax * 12 * nc * 8));
    RET(ensure(ctx, ctx->c32, (size_t)nmax * 3 * nc * 16));
    RET(ensure(ctx, ctx->clm, (size_t)nmax * nc * 4));
    RET(ensure(ctx, ctx->cn, (size_t)nc * 4));
    RET(ensure(ctx, ctx->cR2, (size_t)nc * 8));
    RET(ensure(ctx, ctx->cr50, (size_t)nc * 8));
    RET(ensure(ctx, ctx->crt, (size_t)nc * 8));
    RET(ensure(ctx, ctx->cname, (size_t)nc * 40));
    CK(cudaMemcpyAsync(ctx->x_ps0.p, p6.data(), p6.size() * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->x_sig21.p, s21.data(), s21.size() * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->x_npts.p, npts_slot.data(), (size_t)nc * 4, cudaMemcpyHostToDevice, ctx->st));
    ctx->stats = PgxStats();
    RET(run_lin(ctx, ctx->st, nc, P<double>(ctx->x_ps0), P<double>(ctx->x_sig21), P<int>(ctx->x_npts), nmax,
                ctx->x_opos, ctx->x_ovel, P<double>(ctx->x_t64), P<float4>(ctx->x_t32), P<float>(ctx->x_lm), false));
    // slot order -> cluster order (a column gather, once per table)
    MRET(pgx::gather_columns(ctx->st, nc, nmax, order.data(), P<double>(ctx->x_t64), P<float4>(ctx->x_t32),
                            P<float>(ctx->x_lm), P<double>(ctx->c64), P<float4>(ctx->c32), P<float>(ctx->clm),
                            ctx->mixed));
    std::vector<double> R2(nc), r50(nc), rt(nc);
    for (int i = 0; i < nc; i++) {
        double R = (r_kernel > 0 ? r_kernel * r50_pc[i] : rtot_pc[i]) / 1000.0;
        R2[i] = R * R;
        r50[i] = r50_pc[i] / 1000.0;
        rt[i] = rtot_pc[i] / 1000.0;
    }
    CK(cudaMemcpyAsync(ctx->cn.p, npts.data(), (size_t)nc * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->cR2.p, R2.data(), (size_t)nc * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->cr50.p, r50.data(), (size_t)nc * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->crt.p, rt.data(), (size_t)nc * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->cname.p, names, (size_t)nc * 40, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->nc = nc;
    ctx->ncp = nmax;
    MRET(pgx::mixed_cluster_aux(ctx->st, nc, nmax, P<int>(ctx->cn), P<double>(ctx->c64), P<double>(ctx->cR2),
                               P<float4>(ctx->c32), P<float>(ctx->clm), ctx->mixed));
    RET(ensure(ctx, ctx->cblk, (size_t)((nmax + pgx::kBlockPoints - 1) / pgx::kBlockPoints) * nc * 64));
    MRET(pgx::block_tables(ctx->st, nc, nmax, P<int>(ctx->cn), P<double>(ctx->c64), P<float>(ctx->clm),
                           P<double>(ctx->cR2), P<float4>(ctx->cblk), ctx->mixed.err));
    if (ctx->scan_tma) {
        ctx->nblk = (nmax + pgx::kBlockPoints - 1) / pgx::kBlockPoints;
        ctx->lm_pitch = (nmax + 3) & ~3;
        RET(ensure(ctx, ctx->cblk_cm, (size_t)ctx->nblk * nc * 64));
        RET(ensure(ctx, ctx->c32_cm, (size_t)nmax * nc * 48));
        RET(ensure(ctx, ctx->clm_cm, (size_t)ctx->lm_pitch * nc * 4));
        RET(ensure(ctx, ctx->werr, 16));
        CK(cudaMemsetAsync(ctx->clm_cm.p, 0, (size_t)ctx->lm_pitch * nc * 4, ctx->st));
        CK(cudaMemsetAsync(ctx->werr.p, 0, 16, ctx->st));
        MRET(pgx::cluster_major(ctx->st, nc, nmax, ctx->nblk, ctx->lm_pitch, P<float4>(ctx->cblk),
                                P<float4>(ctx->c32), P<float>(ctx->clm), P<float4>(ctx->cblk_cm),
                                P<float4>(ctx->c32_cm), P<float>(ctx->clm_cm), ctx->mixed.err));
    }
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pgx_screen_stage(PgxContext *ctx, int nt, const double *ps0, const double *sig, const uint64_t *prefix) {
    if (!ctx) return PGX_E_ARG;
    if (nt <= 0 || !ps0 || !sig || !prefix) return fail(ctx, PGX_E_ARG, "pgx_screen_stage: bad args");
    CK(cudaSetDevice(ctx->device));
    ctx->cur = 0;
    ctx->nparts = 0;
    ctx->trk[1].nt = 0;
    if (ctx->split_min <= 0 || nt < ctx->split_min) return stage_slot(ctx, 0, nt, ps0, sig, prefix, nullptr, ctx->st);
    if (nt > (1 << 20)) return fail(ctx, PGX_E_LIMIT, "pgx_screen_stage: %d stars in one chunk (limit 2^20)", nt);
    // the parts' inputs, SoA per part, back to back: one page-locked staging buffer and one copy
    const double part_stars = std::max(1.0, kPartPairs / std::max(ctx->nc, 1));
    std::vector<int> sizes;
    if (ctx->parts == 0) {
        // parts ramping up: the first of about kPartPairs pairs, each next s + 3s/4 after one of s, a last part under
        // half of the one before merged into that one where the two together stay within that growth, at least two
        int s = std::min(nt, (int)std::lround(part_stars));
        for (int f = 0; f < nt; f += s, s = s + std::max(1, 3 * s / 4)) sizes.push_back(std::min(s, nt - f));
        const size_t k = sizes.size();
        if (k > 2 && 2 * sizes[k - 1] < sizes[k - 2] &&
            sizes[k - 2] + sizes[k - 1] <= sizes[k - 3] + 3 * sizes[k - 3] / 4) {
            sizes[k - 2] += sizes[k - 1];
            sizes.pop_back();
        }
        if (sizes.size() < 2) sizes = {nt / 2, nt - nt / 2};
    } else {
        const int K0 = std::min(nt, ctx->parts);                    // pgx_screen_parts: K equal parts
        for (int p = 0; p < K0; p++) sizes.push_back(nt / K0 + (p < nt % K0 ? 1 : 0));
    }
    const int K = (int)sizes.size();
    ctx->part_n.assign(K, 0);
    ctx->part_off.assign(K, 0);
    ctx->part_at.assign(K, 0);
    size_t bytes = 0;
    for (int p = 0, off = 0; p < K; p++) {
        ctx->part_n[p] = sizes[p];
        ctx->part_off[p] = off;
        ctx->part_at[p] = bytes;
        off += ctx->part_n[p];
        bytes += (size_t)ctx->part_n[p] * (6 + 21 + 1) * 8;
    }
    if (ctx->h_part_cap < bytes) {
        pgx_host_free(ctx->h_part);
        ctx->h_part_cap = 0;
        ctx->h_part = (char *)pgx_host_alloc(bytes);
        if (!ctx->h_part) return fail(ctx, PGX_E_NOMEM, "pgx_screen_stage: %zu bytes of page-locked memory", bytes);
        ctx->h_part_cap = bytes;
    }
    for (int p = 0; p < K; p++) {
        const int n = ctx->part_n[p], o = ctx->part_off[p];
        double *p6 = reinterpret_cast<double *>(ctx->h_part + ctx->part_at[p]), *s21 = p6 + (size_t)6 * n;
        to_soa_into(n, ps0 + (size_t)6 * o, sig + (size_t)36 * o, p6, s21);
        memcpy(s21 + (size_t)21 * n, prefix + o, (size_t)n * 8);
    }
    RET(ensure(ctx, ctx->part_in, bytes));
    CK(cudaMemcpyAsync(ctx->part_in.p, ctx->h_part, bytes, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->nparts = K;
    bind_part(ctx, 0, 0);
    return 0;
}

int pgx_screen_split(PgxContext *ctx, int min_stars) {
    if (!ctx) return PGX_E_ARG;
    if (min_stars < 0) return fail(ctx, PGX_E_ARG, "pgx_screen_split: %d", min_stars);
    ctx->split_min = min_stars;
    return 0;
}

int pgx_screen_parts(PgxContext *ctx, int parts) {
    if (!ctx) return PGX_E_ARG;
    if (parts != 0 && (parts < 2 || parts > 64)) return fail(ctx, PGX_E_ARG, "pgx_screen_parts: %d (0, or 2 to 64)", parts);
    ctx->parts = parts;
    return 0;
}

int pgx_screen_exec(PgxContext *ctx, double tmax_myr, double cut, int precision, long *n_rows) {
    if (!ctx) return PGX_E_ARG;
    if (ctx->nc <= 0) return fail(ctx, PGX_E_ARG, "pgx_screen_exec: no cluster table (pgx_screen_clusters)");
    if (ctx->trk[ctx->cur].nt <= 0) return fail(ctx, PGX_E_ARG, "pgx_screen_exec: no stars staged (pgx_screen_stage)");
    if (!(tmax_myr > 0) || !(cut > 0)) return fail(ctx, PGX_E_ARG, "pgx_screen_exec: tmax %g chi2_max %g", tmax_myr, cut);
    if (precision != PGX_FP64 && precision != PGX_MIXED) return fail(ctx, PGX_E_ARG, "precision %d", precision);
    CK(cudaSetDevice(ctx->device));
    ctx->stats = PgxStats();
    CK(cudaEventRecord(ctx->ev[EV_START], ctx->st));
    if (ctx->nparts == 0) {
        RET(tracks_slot(ctx, ctx->cur, tmax_myr, ctx->st, true));
        RET(screen_slot(ctx, ctx->cur, cut, precision, n_rows, true));
        ctx->stats.parts = 1;
        return 0;
    }
    // a chunk staged in parts: part p is screened from slot p & 1 while, with the mixed screen, part p + 1's orbits
    // run on the side stream in the other slot (FP64 pipe beside FP32 and integer work); the plain FP64 path runs
    // them in turn.  A slot is bound to its next part only after its previous part's screen has returned (the
    // screen ends with a synchronize).  The first part's orbits are the only ones not hidden.
    const int K = ctx->nparts;
    const bool overlap = precision == PGX_MIXED;
    bind_part(ctx, 0, 0);
    RET(tracks_slot(ctx, 0, tmax_myr, ctx->st, true));
    long rows = 0;
    for (int p = 0; p < K; p++) {
        const int s = p & 1;
        if (p + 1 < K) {
            bind_part(ctx, s ^ 1, p + 1);
            // the second part's orbits start after the first part's: both at once would share the FP64 pipes and
            // hold back the first screen by the second part's orbits too
            if (overlap && p == 0) CK(cudaStreamWaitEvent(ctx->side, ctx->ev[EV_COV], 0));
            if (overlap) RET(tracks_slot(ctx, s ^ 1, tmax_myr, ctx->side, false, kSideOrbitBlocksPerSm * ctx->sms));
        }
        // the first part's screen keeps the exec's stats (its orbit and covariance times); later parts' are added
        const PgxStats acc = ctx->stats;
        if (p > 0) ctx->stats = PgxStats();
        long np = 0;
        RET(screen_slot(ctx, s, cut, precision, &np, true, rows, ctx->part_off[p]));
        if (p > 0) {
            PgxStats &S = ctx->stats;
            S.ms_orbit = acc.ms_orbit;
            S.ms_cov = acc.ms_cov;
            S.ms_scan += acc.ms_scan;
            S.ms_select += acc.ms_select;
            S.ms_finish += acc.ms_finish;
            S.pairs += acc.pairs;
            S.kept += acc.kept;
            S.body_steps += acc.body_steps;
            S.orbit_body_steps = acc.orbit_body_steps;
            S.candidates += acc.candidates;
            S.ambiguous += acc.ambiguous;
            S.rechecked_points += acc.rechecked_points;
            S.rechecked_draws += acc.rechecked_draws;
            S.kernels += acc.kernels;
        }
        rows += np;
        if (!overlap && p + 1 < K) RET(tracks_slot(ctx, s ^ 1, tmax_myr, ctx->st, false));
    }
    ctx->stats.parts = K;
    if (n_rows) *n_rows = rows;
    return 0;
}

int pgx_screen_fetch(PgxContext *ctx, PgxScreenRow *rows, long n) {
    if (!ctx) return PGX_E_ARG;
    if (n < 0 || n > ctx->n_rows || (n > 0 && !rows)) return fail(ctx, PGX_E_ARG, "pgx_screen_fetch: n %ld", n);
    if (n == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(rows, ctx->rows.p, (size_t)n * sizeof(PgxScreenRow), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pgx_screen(PgxContext *ctx, int nt, const double *ps0, const double *sig, const uint64_t *prefix, double tmax,
               double cut, int precision, PgxScreenRow **rows, long *n_rows) {
    if (!ctx) return PGX_E_ARG;
    if (!rows || !n_rows) return fail(ctx, PGX_E_ARG, "pgx_screen: bad args");
    *rows = nullptr;
    *n_rows = 0;
    RET(pgx_screen_stage(ctx, nt, ps0, sig, prefix));
    long n = 0;
    RET(pgx_screen_exec(ctx, tmax, cut, precision, &n));
    PgxScreenRow *r = (PgxScreenRow *)malloc(sizeof(PgxScreenRow) * (n > 0 ? n : 1));
    if (!r) return fail(ctx, PGX_E_NOMEM, "pgx_screen: host allocation of %ld rows", n);
    int rc = pgx_screen_fetch(ctx, r, n);
    if (rc) {
        free(r);
        return rc;
    }
    *rows = r;
    *n_rows = n;
    return 0;
}

int pgx_screen_into(PgxContext *ctx, int nt, const double *ps0, const double *sig, const uint64_t *prefix,
                    double tmax, double cut, int precision, PgxScreenRow *rows, long cap, long *n_rows) {
    if (!ctx) return PGX_E_ARG;
    if (!n_rows || cap < 0 || (cap > 0 && !rows)) return fail(ctx, PGX_E_ARG, "pgx_screen_into: bad args");
    *n_rows = 0;
    RET(pgx_screen_stage(ctx, nt, ps0, sig, prefix));
    long n = 0;
    RET(pgx_screen_exec(ctx, tmax, cut, precision, &n));
    *n_rows = n;
    if (n > cap) return fail(ctx, PGX_E_LIMIT, "pgx_screen_into: %ld rows, room for %ld", n, cap);
    return pgx_screen_fetch(ctx, rows, n);
}

}  // extern "C"

namespace {
// Rows or text out of the chunk pipeline (pgx_screen_chunks, pgx_screen_chunks_text).
struct ChunkOut {
    int (*rows)(void *arg, int first, const PgxScreenRow *rows, long n) = nullptr;
    int (*text)(void *arg, int first, const char *text, size_t bytes, long n_rows) = nullptr;
    void *arg = nullptr;
};

// Four stages run at once: the host draws of chunk c + 2 (a helper thread); the orbits of chunk c + 1 on the
// high-priority side stream, whose FP64 work shares the SMs with the FP32 and integer work of the screen of chunk c
// on the main stream (both issued by a worker thread, which then copies the rows into device slot c % 2 -- or
// formats them there as text -- and from there to page-locked host memory on a copy stream); and the output of
// chunk c - 1 on the calling thread.  Track slot c % 2 and output slot c % 2 are reused for chunk c + 2 only after
// chunk c is screened and its output has returned.
int screen_pipeline(PgxContext *ctx, const PhTarget *t, int nt, int chunk, int n_samp, int threads, double tmax,
                    double cut, int precision, const ChunkOut &out) {
    const bool text = out.text != nullptr;
    CK(cudaSetDevice(ctx->device));
    const int th = threads > 0 ? threads : pgh_default_threads();
    // Chunk boundaries: `chunk` stars each, except that the first chunks ramp up from about kPartPairs star-cluster
    // pairs, each half again as large as the last: the first chunk's orbits are the only ones not traced beside
    // another chunk's screen, and each later chunk's orbits (FP64, at least one warp's 2,000 steps long) stay shorter
    // than the screen before them.  Measured on 8 chunks of 20,000 stars x 4,087 clusters: 82.5-87.8 against
    // 87.1-90.6 ms per chunk without the ramp, 84.2-89.6 when doubling.
    std::vector<int> cfirst;
    {
        int s = std::min(chunk, std::max(1, (int)std::lround(kPartPairs / std::max(ctx->nc, 1))));
        for (int f = 0; f < nt; f += s, s = std::min(chunk, s + std::max(1, s / 2))) cfirst.push_back(f);
        cfirst.push_back(nt);
    }
    const int nch = (int)cfirst.size() - 1;
    struct Draw {
        std::vector<double> ps0, sig;
        std::vector<uint64_t> pre;
        std::vector<char> ids;
        int first = 0, n = 0;
    } buf[2];
    for (auto &b : buf) {
        b.ps0.resize((size_t)6 * chunk);
        b.sig.resize((size_t)36 * chunk);
        b.pre.resize(chunk);
        if (text) b.ids.resize((size_t)40 * chunk);
    }
    auto draw = [&](int c, Draw &b) {
        b.first = cfirst[c];
        b.n = cfirst[c + 1] - cfirst[c];
        pgh_draw_targets(t + b.first, b.n, n_samp, th, b.ps0.data(), b.sig.data(), b.pre.data());
        for (int i = 0; text && i < b.n; i++) memcpy(&b.ids[(size_t)40 * i], t[b.first + i].id, 40);
    };
    cudaStream_t cs = nullptr;
    cudaEvent_t ev_rows[2] = {}, ev_host[2] = {};
    CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = 0;
    for (int i = 0; i < 2 && rc == 0; i++) {
        if (cudaEventCreateWithFlags(&ev_rows[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_host[i], cudaEventDisableTiming) != cudaSuccess)
            rc = fail(ctx, PGX_E_CUDA, "screen chunks: events");
    }
    std::mutex mu;
    std::condition_variable cv;
    int produced = 0, consumed = 0, worker_rc = 0;
    bool worker_done = false, stop = false;
    long n_of[2] = {0, 0};
    size_t bytes_of[2] = {0, 0};
    int first_of[2] = {0, 0};
    // host buffer of slot s with room for `bytes` (page-locked, grown by a quarter)
    auto host_room = [&](int s, size_t bytes) {
        if (ctx->h_cap[s] >= bytes) return 0;
        pgx_host_free(ctx->h_buf[s]);
        ctx->h_cap[s] = 0;
        const size_t cap = bytes + bytes / 4 + 65536;
        ctx->h_buf[s] = (char *)pgx_host_alloc(cap);
        if (!ctx->h_buf[s]) return fail(ctx, PGX_E_NOMEM, "screen chunks: %zu bytes of page-locked memory", cap);
        ctx->h_cap[s] = cap;
        return 0;
    };
    // chunk c's draws into buf[c % 2], staged into track slot c % 2 and its orbits started on the side stream
    auto start_tracks = [&](int c) {
        const Draw &b = buf[c & 1];
        int r = stage_slot(ctx, c & 1, b.n, b.ps0.data(), b.sig.data(), b.pre.data(), text ? b.ids.data() : nullptr,
                           ctx->side);
        const int blocks = c == 0 ? 0 : kSideOrbitBlocksPerSm * ctx->sms;     // chunk 0 has the GPU to itself
        return r ? r : tracks_slot(ctx, c & 1, tmax, ctx->side, false, blocks);
    };
    auto worker = [&]() {
        int wrc = cudaSetDevice(ctx->device) == cudaSuccess ? 0 : fail(ctx, PGX_E_CUDA, "screen chunks: device");
        std::thread ahead;
        if (wrc == 0) {
            draw(0, buf[0]);
            wrc = start_tracks(0);
            if (nch > 1) ahead = std::thread(draw, 1, std::ref(buf[1]));
        }
        for (int c = 0; c < nch && wrc == 0; c++) {
            const int first = cfirst[c];
            if (c + 1 < nch) {                            // the next chunk's orbits, beside this chunk's screen
                ahead.join();
                wrc = start_tracks(c + 1);
                if (wrc == 0 && c + 2 < nch) ahead = std::thread(draw, c + 2, std::ref(buf[c & 1]));
            }
            long n = 0;
            if (wrc == 0) wrc = screen_slot(ctx, c & 1, cut, precision, &n, false);
            const int slot = c & 1;
            if (wrc == 0) {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return consumed >= c - 1 || stop; });
                if (stop) wrc = -1;
            }
            size_t bytes = (size_t)n * sizeof(PgxScreenRow);
            Buf &dev = ctx->rows_b[slot];
            if (wrc == 0 && text && n > 0) {
                // the lines formatted into the device slot (the star ids came with the chunk's inputs)
                const pgx::TextLabels L = {P<char>(ctx->trk[c & 1].ids), P<char>(ctx->lab_names),
                                           P<char>(ctx->lab_kinds), P<double>(ctx->lab_age16),
                                           P<double>(ctx->lab_age84)};
                for (int attempt = 0; wrc == 0 && attempt < 2; attempt++) {
                    std::string err;
                    size_t need = 0;
                    const int frc = pgx::format_rows(ctx->st, n, P<pgx::ScreenRowDev>(ctx->rows), L, ctx->text_bufs,
                                                     P<char>(dev), dev.cap, &need, err);
                    if (frc == 0) {
                        bytes = need;
                        break;
                    }
                    if (frc != PGX_E_LIMIT || attempt == 1) wrc = fail(ctx, frc, "row text: %s", err.c_str());
                    else wrc = ensure(ctx, dev, need);
                }
            } else if (wrc == 0 && n > 0) {
                wrc = ensure(ctx, dev, bytes);
                if (wrc == 0 && cudaMemcpyAsync(dev.p, ctx->rows.p, bytes, cudaMemcpyDeviceToDevice, ctx->st) !=
                                    cudaSuccess)
                    wrc = fail(ctx, PGX_E_CUDA, "screen chunks: row copy");
            }
            if (wrc == 0) wrc = host_room(slot, bytes);
            if (wrc == 0 && n > 0) {
                const cudaError_t e[3] = {cudaEventRecord(ev_rows[slot], ctx->st),
                                          cudaStreamWaitEvent(cs, ev_rows[slot], 0),
                                          cudaMemcpyAsync(ctx->h_buf[slot], dev.p, bytes, cudaMemcpyDeviceToHost, cs)};
                for (cudaError_t x : e)
                    if (x != cudaSuccess && wrc == 0)
                        wrc = fail(ctx, PGX_E_CUDA, "screen chunks: copy to the host: %s", cudaGetErrorString(x));
            }
            if (wrc == 0 && cudaEventRecord(ev_host[slot], cs) != cudaSuccess)
                wrc = fail(ctx, PGX_E_CUDA, "screen chunks: event record");
            if (wrc == 0) {
                std::lock_guard<std::mutex> lk(mu);
                n_of[slot] = n;
                bytes_of[slot] = n > 0 ? bytes : 0;
                first_of[slot] = first;
                produced = c + 1;
                cv.notify_all();
            }
        }
        if (ahead.joinable()) ahead.join();
        cudaStreamSynchronize(ctx->side);                 // no orbits left running on a slot after an early stop
        std::lock_guard<std::mutex> lk(mu);
        worker_rc = wrc;
        worker_done = true;
        cv.notify_all();
    };
    std::thread gpu;
    if (rc == 0) gpu = std::thread(worker);
    for (int c = 0; c < nch && rc == 0; c++) {
        long n;
        size_t bytes;
        int first;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return produced > c || worker_done; });
            if (produced <= c) break;                     // the worker stopped: its code is returned below
            n = n_of[c & 1];
            bytes = bytes_of[c & 1];
            first = first_of[c & 1];
        }
        const char *h = ctx->h_buf[c & 1];
        if (cudaEventSynchronize(ev_host[c & 1]) != cudaSuccess) rc = PGX_E_CUDA;
        else if (text ? out.text(out.arg, first, h, bytes, n)
                      : out.rows(out.arg, first, reinterpret_cast<const PgxScreenRow *>(h), n))
            rc = PGX_E_ARG;
        std::lock_guard<std::mutex> lk(mu);
        consumed = c + 1;
        if (rc) stop = true;
        cv.notify_all();
    }
    if (gpu.joinable()) gpu.join();
    // the slots hold pipeline chunks now, not a pgx_screen_stage chunk
    ctx->nparts = 0;
    ctx->trk[0].nt = ctx->trk[1].nt = 0;
    // codes set here, after the worker has ended, so that the message is this function's
    if (rc == PGX_E_ARG) rc = fail(ctx, PGX_E_ARG, "screen chunks: the output callback stopped the run");
    else if (rc == PGX_E_CUDA) rc = fail(ctx, PGX_E_CUDA, "screen chunks: copy to the host failed");
    else if (rc == 0 && worker_rc > 0) rc = worker_rc;
    cudaStreamSynchronize(cs);
    for (int i = 0; i < 2; i++) {
        if (ev_rows[i]) cudaEventDestroy(ev_rows[i]);
        if (ev_host[i]) cudaEventDestroy(ev_host[i]);
    }
    cudaStreamDestroy(cs);
    return rc;
}
}  // namespace

extern "C" {

int pgx_screen_chunks(PgxContext *ctx, const PhTarget *t, int nt, int chunk, int n_samp, int threads, double tmax,
                      double cut, int precision, int (*emit)(void *arg, int first, const PgxScreenRow *rows, long n),
                      void *arg) {
    if (!ctx) return PGX_E_ARG;
    if (nt < 0 || (nt > 0 && !t) || chunk <= 0 || chunk > (1 << 20) || n_samp < 0 || !emit)
        return fail(ctx, PGX_E_ARG, "pgx_screen_chunks: bad args");
    if (nt == 0) return 0;
    ChunkOut out;
    out.rows = emit;
    out.arg = arg;
    return screen_pipeline(ctx, t, nt, chunk, n_samp, threads, tmax, cut, precision, out);
}

int pgx_screen_chunks_text(PgxContext *ctx, const PhTarget *t, int nt, const PhCluster *cl, int nc, int chunk,
                           int n_samp, int threads, double tmax, double cut, int precision,
                           int (*emit)(void *arg, int first, const char *text, size_t bytes, long n_rows), void *arg) {
    if (!ctx) return PGX_E_ARG;
    if (nt < 0 || (nt > 0 && !t) || !cl || nc != ctx->nc || chunk <= 0 || chunk > (1 << 20) || n_samp < 0 || !emit)
        return fail(ctx, PGX_E_ARG, "pgx_screen_chunks_text: bad args (%d clusters given, %d resident)", nc, ctx->nc);
    if (nt == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    // the clusters' labels: name, kind, age16, age84
    std::vector<char> names((size_t)40 * nc), kinds(nc);
    std::vector<double> a16(nc), a84(nc);
    for (int i = 0; i < nc; i++) {
        memcpy(&names[(size_t)40 * i], cl[i].name, 40);
        kinds[i] = cl[i].kind;
        a16[i] = cl[i].age16;
        a84[i] = cl[i].age84;
    }
    RET(ensure(ctx, ctx->lab_names, names.size()));
    RET(ensure(ctx, ctx->lab_kinds, kinds.size()));
    RET(ensure(ctx, ctx->lab_age16, (size_t)8 * nc));
    RET(ensure(ctx, ctx->lab_age84, (size_t)8 * nc));
    CK(cudaMemcpy(ctx->lab_names.p, names.data(), names.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->lab_kinds.p, kinds.data(), kinds.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->lab_age16.p, a16.data(), (size_t)8 * nc, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->lab_age84.p, a84.data(), (size_t)8 * nc, cudaMemcpyHostToDevice));
    ChunkOut out;
    out.text = emit;
    out.arg = arg;
    return screen_pipeline(ctx, t, nt, chunk, n_samp, threads, tmax, cut, precision, out);
}

void *pgx_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
    return p;
}

void pgx_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

namespace {
// the clone kernels' cap on blocks per SM for a launch now (0: none): the static one, or, with a busy flag, the cap
// while the flag is set
int mc_cap_now(const PgxContext *ctx) {
    if (!ctx->mc_busy) return ctx->mc_blocks_per_sm;
    return __atomic_load_n(ctx->mc_busy, __ATOMIC_ACQUIRE) != 0 ? ctx->mc_blocks_per_sm : 0;
}

// the captured prep + trace + reduce sequence of clone-kernel variant v (parameters read from ctx->p_params), with the
// grid capped when `capped` (a live cap keeps one graph of each kind)
int mc_graph(PgxContext *ctx, int v, bool capped, cudaGraphExec_t &exec) {
    cudaGraphExec_t &slot = capped ? ctx->mc_exec_capped[v] : ctx->mc_exec[v];
    if (slot) {
        exec = slot;
        return 0;
    }
    RET(ensure(ctx, ctx->p_params, sizeof(pgx::McPairs)));
    int grid = 0;
    CK(pgx::mc_variant_grid(v, ctx->sms, grid));
    if (capped) grid = std::min(grid, ctx->mc_blocks_per_sm * ctx->sms);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    const cudaError_t le = pgx::launch_mc(v, grid, ctx->sms * 4, ctx->sms * 8, ctx->st,
                                          P<pgx::McPairs>(ctx->p_params));
    const cudaError_t ce = cudaStreamEndCapture(ctx->st, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(ctx, PGX_E_CUDA, "clone graph capture: %s", cudaGetErrorString(le != cudaSuccess ? le : ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&slot, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(ctx, PGX_E_CUDA, "clone graph instantiate: %s", cudaGetErrorString(ie));
    exec = slot;
    return 0;
}

int pair_run(PgxContext *ctx, int variant, int n_pairs, const int *clone_off, const double *ps, const int *steps,
             const double *dt, const double *r50_pc, const double *rtot_pc, PhResult *res, double *clone_out) {
    if (!ctx) return PGX_E_ARG;
    if (n_pairs < 0 || (n_pairs > 0 && (!clone_off || !steps || !dt || !r50_pc || !rtot_pc || !res)))
        return fail(ctx, PGX_E_ARG, "pgx_pair: bad args");
    if (n_pairs == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    const int M = clone_off[n_pairs];
    if (clone_off[0] != 0 || M < 0 || (M > 0 && !ps)) return fail(ctx, PGX_E_ARG, "pgx_pair: clone_off");
    int warps = 4, cpl = 1, minb = 1;
    pgx::mc_variant_shape(variant, warps, cpl, minb);
    int mmax = 0;
    for (int p = 0; p < n_pairs; p++) {
        const int m = clone_off[p + 1] - clone_off[p];
        if (m < 0) return fail(ctx, PGX_E_ARG, "pgx_pair: clone_off not ascending at %d", p);
        if (m > pgx::kMaxPairClones)
            return fail(ctx, PGX_E_LIMIT, "pgx_pair: pair %d has %d clones (limit %d)", p, m, pgx::kMaxPairClones);
        if (steps[p] < 0) return fail(ctx, PGX_E_ARG, "pgx_pair: steps[%d] = %d", p, steps[p]);
        mmax = std::max(mmax, m);
    }
    // pairs of at most 1024 clones (every batch of the benchmark and serving workloads) run the captured
    // prep + trace + reduce graph; bigger pairs the fused kernel and the block-wide reduction
    const bool graph = mmax <= 1024;
    const int chunk = graph ? 32 * cpl : 32;
    std::vector<int4> items;
    int big_n2 = 0;
    long long clone_steps = 0;
    for (int p = 0; p < n_pairs; p++) {
        const int m = clone_off[p + 1] - clone_off[p];
        if (m > 1024 && m <= pgx::kSortMax) {
            int n2 = 1;
            while (n2 < m) n2 <<= 1;
            big_n2 = std::max(big_n2, n2);
        }
        for (int c0 = 0; c0 < m; c0 += chunk)
            items.push_back(make_int4(p, clone_off[p] + c0, std::min(chunk, m - c0), 0));
        clone_steps += (long long)m * steps[p];
    }
    std::stable_sort(items.begin(), items.end(), [&](const int4 &a, const int4 &b) { return steps[a.x] > steps[b.x]; });
    RET(ensure(ctx, ctx->p_off, (size_t)(n_pairs + 1) * 4));
    RET(ensure(ctx, ctx->p_ps, (size_t)M * 12 * 8));
    RET(ensure(ctx, ctx->p_steps, (size_t)n_pairs * 4));
    RET(ensure(ctx, ctx->p_dt, (size_t)n_pairs * 8));
    RET(ensure(ctx, ctx->p_r50, (size_t)n_pairs * 8));
    RET(ensure(ctx, ctx->p_rt, (size_t)n_pairs * 8));
    RET(ensure(ctx, ctx->p_items, items.size() * sizeof(int4)));
    RET(ensure(ctx, ctx->p_q, 16));
    RET(ensure(ctx, ctx->p_done, (size_t)n_pairs * 4));
    RET(ensure(ctx, ctx->p_cres, (size_t)M * 3 * 8));
    RET(ensure(ctx, ctx->p_res, (size_t)n_pairs * sizeof(PhResult)));
    CK(cudaMemcpyAsync(ctx->p_off.p, clone_off, (size_t)(n_pairs + 1) * 4, cudaMemcpyHostToDevice, ctx->st));
    if (M > 0) CK(cudaMemcpyAsync(ctx->p_ps.p, ps, (size_t)M * 12 * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->p_steps.p, steps, (size_t)n_pairs * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->p_dt.p, dt, (size_t)n_pairs * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->p_r50.p, r50_pc, (size_t)n_pairs * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->p_rt.p, rtot_pc, (size_t)n_pairs * 8, cudaMemcpyHostToDevice, ctx->st));
    if (!items.empty())
        CK(cudaMemcpyAsync(ctx->p_items.p, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->st));
    pgx::McPairs Pp;
    Pp.n_pairs = n_pairs; Pp.n_clones = M; Pp.n_items = (int)items.size();
    Pp.clone_off = P<int>(ctx->p_off); Pp.ps = P<double>(ctx->p_ps); Pp.steps = P<int>(ctx->p_steps);
    Pp.dt = P<double>(ctx->p_dt); Pp.r50_pc = P<double>(ctx->p_r50); Pp.rtot_pc = P<double>(ctx->p_rt);
    Pp.items = P<int4>(ctx->p_items); Pp.qhead = P<int>(ctx->p_q); Pp.done = P<int>(ctx->p_done);
    Pp.cres = P<double>(ctx->p_cres); Pp.res = P<pgx::PhResultDev>(ctx->p_res);
    ctx->stats = PgxStats();
    if (graph) {
        cudaGraphExec_t exec;
        RET(mc_graph(ctx, variant, mc_cap_now(ctx) > 0, exec));
        // the parameters travel by copy: the graph's kernels read them from p_params
        CK(cudaMemcpyAsync(ctx->p_params.p, &Pp, sizeof Pp, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaEventRecord(ctx->ev[EV_PAIR0], ctx->st));
        CK(cudaGraphLaunch(exec, ctx->st));
        ctx->stats.kernels += 3;
    } else {
        CK(cudaMemsetAsync(ctx->p_q.p, 0, 16, ctx->st));
        CK(cudaMemsetAsync(ctx->p_done.p, 0, (size_t)n_pairs * 4, ctx->st));
        CK(cudaEventRecord(ctx->ev[EV_PAIR0], ctx->st));
        if (!items.empty()) {
            int per_sm = 0;
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pgx::k_pair_mc, pgx::kMcThreads, 0));
            const int warps_needed = (int)items.size();
            int grid = std::max(1, ctx->sms * std::max(1, per_sm));
            const int cap = mc_cap_now(ctx);
            if (cap > 0) grid = std::min(grid, cap * ctx->sms);
            grid = std::min(grid, (warps_needed + pgx::kMcThreads / 32 - 1) / (pgx::kMcThreads / 32));
            pgx::k_pair_mc<<<grid, pgx::kMcThreads, 0, ctx->st>>>(Pp);
            CKL();
            ctx->stats.kernels++;
        }
        const size_t smem = (size_t)big_n2 * 8;
        if (smem > 48 * 1024)
            CK(cudaFuncSetAttribute(pgx::k_pair_reduce_big, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        pgx::k_pair_reduce_big<<<n_pairs, 256, smem, ctx->st>>>(Pp);
        CKL();
        ctx->stats.kernels++;
    }
    CK(cudaEventRecord(ctx->ev[EV_PAIR1], ctx->st));
    CK(cudaMemcpyAsync(res, ctx->p_res.p, (size_t)n_pairs * sizeof(PhResult), cudaMemcpyDeviceToHost, ctx->st));
    if (clone_out && M > 0)
        CK(cudaMemcpyAsync(clone_out, ctx->p_cres.p, (size_t)M * 3 * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->stats.ms_pair = elapsed(ctx, EV_PAIR0, EV_PAIR1);
    ctx->stats.ms_total = ctx->stats.ms_pair;
    ctx->stats.clones = M;
    ctx->stats.clone_steps = clone_steps;
    ctx->stats.body_steps = 2 * clone_steps;
    ctx->stats.pairs = n_pairs;
    return 0;
}
}  // namespace

int pgx_pair(PgxContext *ctx, int n_pairs, const int *clone_off, const double *ps, const int *steps, const double *dt,
             const double *r50_pc, const double *rtot_pc, PhResult *res, double *clone_out) {
    if (!ctx) return PGX_E_ARG;
    return pair_run(ctx, ctx->mc_variant, n_pairs, clone_off, ps, steps, dt, r50_pc, rtot_pc, res, clone_out);
}

int pgx_pair_targets(PgxContext *ctx, int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c, const int *ci,
                     const int *n_clones, double dt_myr, int threads, int batch_pairs, PhResult *res) {
    if (!ctx) return PGX_E_ARG;
    if (n_pairs < 0 || (n_pairs > 0 && (!t || !ti || !c || !ci || !n_clones || !res)) || !(dt_myr > 0))
        return fail(ctx, PGX_E_ARG, "pgx_pair_targets: bad args");
    if (n_pairs == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    const int bp = batch_pairs > 0 ? batch_pairs : 1024, nb = (n_pairs + bp - 1) / bp;
    const int th = threads > 0 ? threads : pgh_default_threads();
    // batch k's clones are drawn into buffer k % 2 (by a helper thread for k > 0) while the GPU traces batch k - 1
    struct Batch {
        std::vector<int> off, steps;
        std::vector<double> dt, r50, rt;
        int p0 = 0, n = 0, rc = 0;
    } b[2];
    auto draw = [&](int k, int i) {
        Batch &x = b[i];
        x.p0 = k * bp;
        x.n = std::min(bp, n_pairs - x.p0);
        long clones = 0;
        for (int q = x.p0; q < x.p0 + x.n; q++) clones += std::max(n_clones[q], 0);
        const size_t need = (size_t)12 * std::max(clones, 1L) * sizeof(double);
        if (ctx->h_clones_cap[i] < need) {
            pgx_host_free(ctx->h_clones[i]);
            ctx->h_clones_cap[i] = 0;
            ctx->h_clones[i] = (double *)pgx_host_alloc(need + need / 4);
            if (!ctx->h_clones[i]) {
                x.rc = -1;
                return;
            }
            ctx->h_clones_cap[i] = need + need / 4;
        }
        x.off.resize(x.n + 1);
        x.steps.resize(x.n);
        x.dt.resize(x.n);
        x.r50.resize(x.n);
        x.rt.resize(x.n);
        x.rc = pgh_draw_pair_batch(x.n, t, ti + x.p0, c, ci + x.p0, n_clones + x.p0, dt_myr, th, x.off.data(),
                                   ctx->h_clones[i], x.steps.data(), x.dt.data(), x.r50.data(), x.rt.data());
    };
    draw(0, 0);
    PgxStats sum = PgxStats();
    int rc = 0;
    for (int k = 0; k < nb && rc == 0; k++) {
        const int i = k & 1;
        std::thread ahead;
        if (k + 1 < nb) ahead = std::thread(draw, k + 1, i ^ 1);
        const Batch &x = b[i];
        if (x.rc) {
            rc = fail(ctx, x.rc == -1 ? PGX_E_NOMEM : PGX_E_LIMIT, "pgx_pair_targets: clone draws of pairs %d..%d",
                      x.p0, x.p0 + x.n);
        } else {
            rc = pair_run(ctx, ctx->mc_variant, x.n, x.off.data(), ctx->h_clones[i], x.steps.data(), x.dt.data(),
                          x.r50.data(), x.rt.data(), res + x.p0, nullptr);
            const PgxStats &st = ctx->stats;
            sum.ms_pair += st.ms_pair;
            sum.clones += st.clones;
            sum.clone_steps += st.clone_steps;
            sum.body_steps += st.body_steps;
            sum.pairs += st.pairs;
            sum.kernels += st.kernels;
        }
        if (ahead.joinable()) ahead.join();
    }
    sum.ms_total = sum.ms_pair;
    ctx->stats = sum;
    return rc;
}

int pgx_screen_shapes(int n, int *min_blocks) {
    const int k = pgx::scan_shapes();
    for (int v = 0; v < n && v < k && min_blocks; v++) min_blocks[v] = pgx::scan_shape(v);
    return k;
}

int pgx_tune_screen(PgxContext *ctx, double tmax_myr, double chi2_max, double *ms, int *best) {
    if (!ctx) return PGX_E_ARG;
    if (!ctx->scan_blocks) return fail(ctx, PGX_E_ARG, "pgx_tune_screen: the block filter is off (PHYGAS_SCAN_BLOCKS)");
    const int k = pgx::scan_shapes();
    int b = 0;
    double bms = 0.0;
    long rows0 = -1;
    for (int v = 0; v < k; v++) {
        ctx->mixed.scan_variant = v;
        long n = 0;
        // twice: the first run of a shape loads its code
        RET(pgx_screen_exec(ctx, tmax_myr, chi2_max, PGX_MIXED, &n));
        RET(pgx_screen_exec(ctx, tmax_myr, chi2_max, PGX_MIXED, &n));
        const double t = ctx->stats.ms_scan;
        if (ms) ms[v] = t;
        if (rows0 < 0) rows0 = n;
        if (n != rows0) return fail(ctx, PGX_E_CUDA, "pgx_tune_screen: shape %d kept %ld pairs, shape 0 %ld", v, n, rows0);
        if (v == 0 || t < bms) { b = v; bms = t; }
    }
    ctx->mixed.scan_variant = b;
    if (best) *best = b;
    return 0;
}

int pgx_tune_pair(PgxContext *ctx, int n_pairs, const int *clone_off, const double *ps, const int *steps,
                  const double *dt, const double *r50_pc, const double *rtot_pc, double *ms, int *best) {
    if (!ctx) return PGX_E_ARG;
    if (n_pairs <= 0) return fail(ctx, PGX_E_ARG, "pgx_tune_pair: empty batch");
    const int nv = pgx::mc_variants();
    std::vector<PhResult> ref(n_pairs), got(n_pairs);
    int b = 0;
    double bms = 0;
    for (int v = 0; v < nv; v++) {
        PhResult *out = v == 0 ? ref.data() : got.data();
        // twice: the first run of a shape also captures and instantiates its graph
        RET(pair_run(ctx, v, n_pairs, clone_off, ps, steps, dt, r50_pc, rtot_pc, out, nullptr));
        RET(pair_run(ctx, v, n_pairs, clone_off, ps, steps, dt, r50_pc, rtot_pc, out, nullptr));
        const double t = ctx->stats.ms_pair;
        if (ms) ms[v] = t;
        if (v > 0 && memcmp(ref.data(), got.data(), sizeof(PhResult) * (size_t)n_pairs) != 0)
            return fail(ctx, PGX_E_CUDA, "pgx_tune_pair: launch shape %d changed the results", v);
        if (v == 0 || t < bms) { b = v; bms = t; }
    }
    ctx->mc_variant = b;
    if (best) *best = b;
    return 0;
}

int pgx_pair_blocks_while(PgxContext *ctx, int blocks_per_sm, const int *busy) {
    if (!ctx) return PGX_E_ARG;
    if (blocks_per_sm < 0) return fail(ctx, PGX_E_ARG, "pgx_pair_blocks: %d", blocks_per_sm);
    CK(cudaSetDevice(ctx->device));
    ctx->mc_blocks_per_sm = blocks_per_sm;
    ctx->mc_busy = busy;
    for (auto *set : {ctx->mc_exec, ctx->mc_exec_capped})   // captured with the old grid
        for (int v = 0; v < 16; v++)
            if (set[v]) {
                cudaGraphExecDestroy(set[v]);
                set[v] = nullptr;
            }
    return 0;
}

int pgx_pair_blocks(PgxContext *ctx, int blocks_per_sm) { return pgx_pair_blocks_while(ctx, blocks_per_sm, nullptr); }

int pgx_pair_shapes(int n, int *warps, int *clones_per_lane, int *min_blocks) {
    const int nv = pgx::mc_variants();
    for (int v = 0; v < n && v < nv; v++) pgx::mc_variant_shape(v, warps[v], clones_per_lane[v], min_blocks[v]);
    return nv;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------------------
// The GPU half of the drop-in API (include/phygas.h).  These per-object / per-pair calls keep the reference's
// signatures and ownership rules; each one runs the same kernels as the batched entry points on a process-wide
// default context.  The reference API has no error channel: a GPU failure here prints the cause and ends the
// process with status 1, as the reference GPU application does (src/main_phygas_boinc.cpp:23-27).
namespace {

PgxContext *g_ctx = nullptr;
std::mutex g_mu;

[[noreturn]] void die(const char *what, const char *why) {
    fprintf(stderr, "phygas_gb300: %s failed: %s\n", what, why);
    fflush(stderr);
    exit(1);
}

PgxContext *dctx() {
    if (!g_ctx) {
        int rc = pgx_open(-1, &g_ctx);
        if (rc) die("pgx_open", rc == PGX_E_NODEV ? "no CUDA device" : "device set-up");
    }
    return g_ctx;
}

void lin_one(PgxContext *ctx, const double ps0[6], const double sig[36], double tmax, PhLin *out) {
    int n = npts_of(tmax);
    out->n = n;
    out->pos = (Vec3 *)malloc(sizeof(Vec3) * n);
    out->vel = (Vec3 *)malloc(sizeof(Vec3) * n);
    out->S = (double(*)[6])malloc(sizeof(double[6]) * n);
    if (pgx_lin(ctx, 1, ps0, sig, &n, &out->pos[0].x, &out->vel[0].x, &out->S[0][0])) die("ph_lin", ctx->err.c_str());
}

// one (star, cluster) pair as a 1 x 1 screen
int pair_tables(PgxContext *ctx, const PhLin *tl, const PhLin *cl, const PhCluster *c, uint64_t seed,
                pgx::ScreenTables &T) {
    const int nmax = std::max(tl->n, cl->n);
    std::vector<double> h((size_t)2 * nmax * 12, 0.0);
    auto pack = [&](const PhLin *l, double *dst) {
        for (int k = 0; k < l->n; k++) {
            double *o = dst + (size_t)k * 12;
            o[0] = l->pos[k].x; o[1] = l->pos[k].y; o[2] = l->pos[k].z;
            o[3] = l->vel[k].x; o[4] = l->vel[k].y; o[5] = l->vel[k].z;
            for (int i = 0; i < 6; i++) o[6 + i] = l->S[k][i];
        }
    };
    pack(tl, h.data());
    pack(cl, h.data() + (size_t)nmax * 12);
    const double R = (ph_screen_r > 0 ? ph_screen_r * c->r50_pc : c->rtot_pc) / 1000.0;
    struct {
        double R2, r50, rt;
        uint64_t seed;
        int cn, pad;
        char name[40];
    } aux = {R * R, c->r50_pc / 1000.0, c->rtot_pc / 1000.0, seed, cl->n, 0, {0}};
    RET(ensure(ctx, ctx->x_t64, h.size() * 8 + sizeof aux));
    char *base = P<char>(ctx->x_t64);
    CK(cudaMemcpyAsync(base, h.data(), h.size() * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(base + h.size() * 8, &aux, sizeof aux, cudaMemcpyHostToDevice, ctx->st));
    const char *a = base + h.size() * 8;
    T.nt = 1; T.ns = tl->n; T.nc = 1; T.ncp = cl->n; T.s_off = 0;
    T.t64 = (const double *)base;
    T.c64 = (const double *)base + (size_t)nmax * 12;
    T.t32 = nullptr; T.c32 = nullptr; T.lm_t = nullptr; T.lm_c = nullptr;
    T.R2 = (const double *)a; T.r50 = (const double *)(a + 8); T.rtot = (const double *)(a + 16);
    T.seed_prefix = (const uint64_t *)(a + 24); T.cn = (const int *)(a + 32); T.cname = a + 40;
    return 0;
}

int chi2_one(PgxContext *ctx, const PhLin *tl, const PhLin *cl, const PhCluster *c, double cut, int *kb, double *sb,
             double *chi2) {
    pgx::ScreenTables T;
    RET(pair_tables(ctx, tl, cl, c, 0, T));
    RET(ensure(ctx, ctx->x_opos, 32));
    double *o = P<double>(ctx->x_opos);
    pgx::k_scan64<<<dim3(1, 1), 32, 0, ctx->st>>>(T, cut, o, (int *)(o + 2), o + 1);
    CKL();
    double hb[3];
    CK(cudaMemcpyAsync(hb, o, sizeof hb, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    *chi2 = hb[0];
    *sb = hb[1];
    memcpy(kb, &hb[2], sizeof(int));
    return 0;
}

int finish_one(PgxContext *ctx, const PhLin *tl, const PhLin *cl, const PhCluster *c, uint64_t seed, double chi2,
               int kb, double sb, PhScreen *res) {
    pgx::ScreenTables T;
    RET(pair_tables(ctx, tl, cl, c, seed, T));
    RET(ensure(ctx, ctx->x_opos, sizeof(pgx::KeptPair) + sizeof(pgx::FinishIn) + sizeof(pgx::ScreenRowDev)));
    char *b = P<char>(ctx->x_opos);
    pgx::KeptPair kp = {0, 0, kb, 0, sb, chi2};
    CK(cudaMemcpyAsync(b, &kp, sizeof kp, cudaMemcpyHostToDevice, ctx->st));
    pgx::FinishIn *fin = (pgx::FinishIn *)(b + sizeof kp);
    pgx::ScreenRowDev *row = (pgx::ScreenRowDev *)(b + sizeof kp + sizeof(pgx::FinishIn));
    pgx::k_finish_prep<<<1, 32, 0, ctx->st>>>(T, 1, (const pgx::KeptPair *)b, fin, row);
    CKL();
    pgx::k_finish64<<<1, 32, 0, ctx->st>>>(1, fin, row);
    CKL();
    pgx::ScreenRowDev r;
    CK(cudaMemcpyAsync(&r, row, sizeof r, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    memset(res, 0, sizeof *res);
    res->chi2 = chi2; res->t = r.t_myr; res->d_nom_pc = r.d_nom_pc; res->sig_pc = r.sig_pc;
    res->p_r50 = r.p_r50; res->p_rtot = r.p_rtot; res->vrel = r.vrel_kms;
    return 0;
}

int reduce_only(PgxContext *ctx, int m, const double *best, const double *tbest, const double *vbest, double r50,
                double rt, PhResult *res) {
    if (m > pgx::kMaxPairClones)
        return fail(ctx, PGX_E_LIMIT, "ph_pair_reduce: %d clones (limit %d)", m, pgx::kMaxPairClones);
    const int off[2] = {0, m};
    RET(ensure(ctx, ctx->p_off, 8));
    RET(ensure(ctx, ctx->p_cres, (size_t)3 * (m > 0 ? m : 1) * 8));
    RET(ensure(ctx, ctx->p_r50, 8));
    RET(ensure(ctx, ctx->p_rt, 8));
    RET(ensure(ctx, ctx->p_res, sizeof(PhResult)));
    CK(cudaMemcpyAsync(ctx->p_off.p, off, 8, cudaMemcpyHostToDevice, ctx->st));
    if (m > 0) {
        CK(cudaMemcpyAsync(P<double>(ctx->p_cres), best, (size_t)m * 8, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaMemcpyAsync(P<double>(ctx->p_cres) + m, tbest, (size_t)m * 8, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaMemcpyAsync(P<double>(ctx->p_cres) + 2 * (size_t)m, vbest, (size_t)m * 8, cudaMemcpyHostToDevice, ctx->st));
    }
    CK(cudaMemcpyAsync(ctx->p_r50.p, &r50, 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->p_rt.p, &rt, 8, cudaMemcpyHostToDevice, ctx->st));
    pgx::McPairs Pp = {};
    Pp.n_pairs = 1; Pp.n_clones = m; Pp.clone_off = P<int>(ctx->p_off); Pp.cres = P<double>(ctx->p_cres);
    Pp.r50_pc = P<double>(ctx->p_r50); Pp.rtot_pc = P<double>(ctx->p_rt); Pp.res = P<pgx::PhResultDev>(ctx->p_res);
    pgx::k_pair_reduce_only<<<1, pgx::kMcThreads, 0, ctx->st>>>(Pp);
    CKL();
    int n2 = 1;
    while (n2 < m) n2 <<= 1;
    const size_t smem = m > 1024 && m <= pgx::kSortMax ? (size_t)n2 * 8 : 0;
    if (smem > 48 * 1024)
        CK(cudaFuncSetAttribute(pgx::k_pair_reduce_big, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pgx::k_pair_reduce_big<<<1, 256, smem, ctx->st>>>(Pp);
    CKL();
    CK(cudaMemcpyAsync(res, ctx->p_res.p, sizeof(PhResult), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

}  // namespace

extern "C" {

void ph_lin_target(const PhTarget *t, double tmax, int n_samp, uint64_t seed, PhLin *out) {
    double ps0[6], sig[36];
    pgh_target_init(t, n_samp, seed, ps0, sig);
    std::lock_guard<std::mutex> lk(g_mu);
    lin_one(dctx(), ps0, sig, tmax, out);
}

void ph_lin_cluster(const PhCluster *c, int n_samp, uint64_t seed, PhLin *out) {
    double ps0[6], sig[36];
    pgh_cluster_init(c, n_samp, seed, ps0, sig);
    std::lock_guard<std::mutex> lk(g_mu);
    lin_one(dctx(), ps0, sig, c->tmax_myr, out);
}

void ph_lin_free(PhLin *l) {
    free(l->pos); free(l->vel); free(l->S);
    l->pos = l->vel = nullptr; l->S = nullptr; l->n = 0;
}

double ph_screen_chi2_cut(const PhLin *tl, const PhLin *cl, const PhCluster *c, double cut, int *kb, double *sb) {
    std::lock_guard<std::mutex> lk(g_mu);
    PgxContext *ctx = dctx();
    double chi2;
    if (chi2_one(ctx, tl, cl, c, cut, kb, sb, &chi2)) die("ph_screen_chi2", ctx->err.c_str());
    return chi2;
}

double ph_screen_chi2(const PhLin *tl, const PhLin *cl, const PhCluster *c, int *kb, double *sb) {
    return ph_screen_chi2_cut(tl, cl, c, INFINITY, kb, sb);
}

void ph_screen_finish(const PhLin *tl, const PhLin *cl, const PhCluster *c, uint64_t seed, double chi2, int kb,
                      double sb, PhScreen *res) {
    std::lock_guard<std::mutex> lk(g_mu);
    PgxContext *ctx = dctx();
    if (finish_one(ctx, tl, cl, c, seed, chi2, kb, sb, res)) die("ph_screen_finish", ctx->err.c_str());
}

void ph_screen(const PhLin *tl, const PhLin *cl, const PhCluster *c, uint64_t seed, PhScreen *res) {
    int kb;
    double sb, chi2 = ph_screen_chi2(tl, cl, c, &kb, &sb);
    ph_screen_finish(tl, cl, c, seed, chi2, kb, sb, res);
}

void ph_pair_clone(const double *ps, int steps, double dt, double *best, double *tbest, double *vbest) {
    std::lock_guard<std::mutex> lk(g_mu);
    PgxContext *ctx = dctx();
    const int off[2] = {0, 1};
    const double r = 0.0;
    PhResult res;
    double out[3];
    if (pgx_pair(ctx, 1, off, ps, &steps, &dt, &r, &r, &res, out)) die("ph_pair_clone", ctx->err.c_str());
    *best = out[0]; *tbest = out[1]; *vbest = out[2];
}

void ph_pair_reduce(const PhCluster *c, int m, const double *best, const double *tbest, const double *vbest,
                    PhResult *res) {
    std::lock_guard<std::mutex> lk(g_mu);
    PgxContext *ctx = dctx();
    if (reduce_only(ctx, m, best, tbest, vbest, c->r50_pc, c->rtot_pc, res)) die("ph_pair_reduce", ctx->err.c_str());
}

void ph_pair(const PhTarget *t, const PhCluster *c, int n_clones, double dt_myr, uint64_t seed, PhResult *res) {
    std::vector<double> ps((size_t)12 * (n_clones > 0 ? n_clones : 1));
    int steps;
    double dt;
    const int m = ph_pair_draw(t, c, n_clones, dt_myr, seed, ps.data(), &steps, &dt);
    const int off[2] = {0, m};
    std::lock_guard<std::mutex> lk(g_mu);
    PgxContext *ctx = dctx();
    if (pgx_pair(ctx, 1, off, ps.data(), &steps, &dt, &c->r50_pc, &c->rtot_pc, res, nullptr))
        die("ph_pair", ctx->err.c_str());
}

}  // extern "C"
