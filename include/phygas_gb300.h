/* phygas_gb300.h -- batched C-ABI of libphygas_gb300 (GB300, sm_103a).
 *
 * The reference's per-pair API (phygas.h) cannot feed a GPU: every call is one star, one pair or one clone.  These
 * entry points take whole chunks and keep their data on the device between stages.  They replace the reference's
 * GPU backend interface, src/phygas_gpu.h:18-31 (pg_init, pg_alloc/put/get/free, pg_lin, pg_chi2, pg_finish,
 * pg_pair), and the loops of its host layer that drive it, src/main_phygas_boinc.cpp:59-301 (gpu_screen, gpu_pair).
 * Plain pointers and sizes only; host buffers in, host buffers out; every call is synchronous on return.
 *
 * Status codes: 0 ok; otherwise one of PGX_E_* below, with a message in pgx_last_error().  (The reference backend
 * returns 0 / 1 with a message on stderr, src/phygas_cuda.cu:16-17.)
 */
#ifndef PHYGAS_GB300_H
#define PHYGAS_GB300_H

#include <stddef.h>
#include <stdint.h>
#include "phygas.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PGX_OK 0
#define PGX_E_ARG 1        /* a size or pointer is invalid */
#define PGX_E_CUDA 2       /* a CUDA call or kernel failed */
#define PGX_E_NOMEM 3      /* device memory exhausted */
#define PGX_E_TIMEOUT 4    /* a bounded wait ran out (pgx_server_wait_for) */
#define PGX_E_LIMIT 5      /* beyond a documented size limit */
#define PGX_E_NODEV 6      /* no usable GPU */
#define PGX_E_PENDING 7    /* pgx_server_query: the job has not finished */

#define PGX_FP64 0         /* the plain FP64 screen */
#define PGX_MIXED 1        /* FP32 screen with FP64 rechecks (identical rows) */

typedef struct PgxContext PgxContext;

/* One device context per GPU: a stream, resident tables and work buffers.  Replaces pg_init
 * (src/phygas_gpu.h:18).  device < 0 picks device 0. */
int pgx_open(int device, PgxContext **ctx);
void pgx_close(PgxContext *ctx);
const char *pgx_last_error(const PgxContext *ctx);
void pgx_free(void *p);              /* frees arrays the pgx_* calls return */

/* State-transition tracks (reference lin_integrate, src/phygas.c:286-323; GPU pg_lin, src/phygas_gpu.h:25):
 * for n objects, nominal phase space ps0[6n], 6x6 initial covariance sig[36n] (row-major), npts[n] points 0.5 Myr
 * apart.  Outputs are the objects' points back to back (object i starts at point sum(npts[0..i-1])): pos[3*],
 * vel[3*], S[6*] (xx xy xz yy yz zz). */
int pgx_lin(PgxContext *ctx, int n, const double *ps0, const double *sig, const int *npts, double *pos, double *vel,
            double *S);

/* ---- stage-1 screen -------------------------------------------------------------------------------------------- */
/* A kept pair (chi2 < chi2_max), in (star, cluster) order: the columns of the reference's rows
 * (src/phygas_screen.c:60-61) plus the argmin point kb and segment fraction sb. */
typedef struct {
    int star, cluster, kb, pad;
    double sb, chi2, t_myr, d_nom_pc, sig_pc, p_r50, p_rtot, vrel_kms;
} PgxScreenRow;

/* Resident cluster table: nominal orbit + 6 neighbours of each cluster integrated on the device (reference
 * ph_lin_cluster, src/phygas.c:336-344); ps0/sig as in pgx_lin, tmax_myr sets each track's length; names (40 bytes
 * each, NUL-terminated) seed the pairs' draws; r_kernel as ph_screen_r (0 = rtot). */
int pgx_screen_clusters(PgxContext *ctx, int nc, const double *ps0, const double *sig, const double *tmax_myr,
                        const double *r50_pc, const double *rtot_pc, const char *names, double r_kernel);

/* Screen nt stars against the resident cluster table (reference ph_lin_target + ph_screen_chi2_cut +
 * ph_screen_finish over every pair, src/phygas_screen.c:50-62; GPU pg_lin + pg_chi2 + pg_finish).
 * ps0/sig as in pgx_lin; seed_prefix[i] = FNV-1a state after "id|" of star i (pgx_seed_prefix), so a pair's seed is
 * ph_seed(id, cluster name); tmax_myr = the star tracks' length (the reference uses the longest cluster tmax).
 * Returns a malloc'ed array of *n_rows rows (free with pgx_free). */
int pgx_screen(PgxContext *ctx, int nt, const double *ps0, const double *sig, const uint64_t *seed_prefix,
               double tmax_myr, double chi2_max, int precision, PgxScreenRow **rows, long *n_rows);

/* The same in three steps, for callers that time the device part alone: stage (host -> device), exec (device
 * only; returns the kept-pair count), fetch (device -> host, n rows into a caller buffer). */
int pgx_screen_stage(PgxContext *ctx, int nt, const double *ps0, const double *sig, const uint64_t *seed_prefix);
int pgx_screen_exec(PgxContext *ctx, double tmax_myr, double chi2_max, int precision, long *n_rows);
int pgx_screen_fetch(PgxContext *ctx, PgxScreenRow *rows, long n);
/* Chunks of at least min_stars stars (default 8192; 0 = never) are staged in parts, and exec traces each part's orbits
 * beside the previous part's screen (the mixed path; the FP64 path screens the parts in turn).  pgx_screen_parts(ctx,
 * K) fixes K equal parts (2 to 64); its default 0 ramps them up: the first of round(1e7 / clusters) stars, each next
 * s + 3s / 4 after one of s stars (integer division), a last part under half of the one before merged into that one
 * where the two together are at most 1.75 times the part before them, at least 2 (20,000 stars at 4,087 clusters:
 * 2,447, 4,282, 7,493, 5,778).  The rows are the same either way. */
int pgx_screen_split(PgxContext *ctx, int min_stars);
int pgx_screen_parts(PgxContext *ctx, int parts);
/* pgx_screen writing into the caller's rows[cap] (no allocation); *n_rows = the kept pairs, PGX_E_LIMIT (rows kept on
 * the device for pgx_screen_fetch) when more than cap.  With rows from pgx_host_alloc the copy runs at the link's
 * full rate: page-locked host memory, allocated once and freed with pgx_host_free. */
int pgx_screen_into(PgxContext *ctx, int nt, const double *ps0, const double *sig, const uint64_t *prefix,
                    double tmax, double chi2_max, int precision, PgxScreenRow *rows, long cap, long *n_rows);
void *pgx_host_alloc(size_t bytes);
/* The whole star list t[nt] in chunks of `chunk` stars, pipelined: while the GPU screens chunk i, the draws of chunk
 * i + 1 (ph_lin_target_init's, on `threads` host threads) run, the rows of chunk i - 1 are copied into page-locked
 * memory on a second stream, and emit(arg, first star of chunk i - 1, rows, count) runs on the calling thread.  The
 * first chunks are smaller where `chunk` is larger than round(1e7 / clusters) stars: the first is that many, each
 * next one s + s / 2 (integer division) after one of s stars, up to `chunk` -- the first chunk's orbits are the only
 * ones not traced beside another chunk's screen.  Star
 * indices in the rows are relative to the chunk's first star; the pointer is valid until emit returns.  Chunks are
 * emitted in order.  A non-zero return from emit stops the run.  The page-locked and device row buffers (two chunks
 * of each) stay with the context for the next call. */
int pgx_screen_chunks(PgxContext *ctx, const PhTarget *t, int nt, int chunk, int n_samp, int threads, double tmax,
                      double chi2_max, int precision,
                      int (*emit)(void *arg, int first, const PgxScreenRow *rows, long n), void *arg);
void pgx_host_free(void *p);
/* pgx_screen_chunks with each chunk's rows as the reference CLI's text lines (src/phygas_screen.c:60-61),
 *   "%s %s %c %.3f %.3f %.2f %.2f %.4f %.4f %.2f %.3f %.3f\n" of target id, cluster name, cluster kind, chi2, t_myr,
 *   d_nom_pc, sig_pc, p_r50, p_rtot, vrel_kms, cluster age16, cluster age84,
 * formatted on the GPU byte for byte as the C library's printf formats them, and handed to
 * emit(arg, first star of the chunk, text, bytes, rows).  cl[nc] are the resident table's clusters, in its order
 * (nc must equal the table's count): the names, kinds and ages of the lines. */
int pgx_screen_chunks_text(PgxContext *ctx, const PhTarget *t, int nt, const PhCluster *cl, int nc, int chunk,
                           int n_samp, int threads, double tmax, double chi2_max, int precision,
                           int (*emit)(void *arg, int first, const char *text, size_t bytes, long n_rows), void *arg);

/* Host draws for the records API (reference ph_lin_target_init / the draws of ph_lin_cluster, src/phygas.c:274-344,
 * seeds ph_seed("lin", id)), on `threads` host threads (<= 0: all cores). */
int pgx_draw_targets(const PhTarget *t, int n, int n_samp, int threads, double *ps0, double *sig,
                     uint64_t *seed_prefix);
int pgx_draw_clusters(const PhCluster *c, int n, int n_samp, int threads, double *ps0, double *sig);
/* The same draws on the GPU (the device-side draws): pgx_draw_targets' outputs for n targets, and
 * pgx_draw_pair_batch's for n_pairs pairs, from the same seeds and random streams (the same draws taken, retries
 * included), with the device's log / exp / sin / cos / sqrt / pow in place of the C library's, so the values agree
 * with the host's within the last bits of those functions rather than bit for bit (the host versions stay the
 * reference's draws exactly).  Host buffers in and out, as the host versions; pgx_stats: ms_total = the draw
 * kernel's device time, clones and pairs for the pair batch. */
int pgx_draw_targets_gpu(PgxContext *ctx, const PhTarget *t, int n, int n_samp, double *ps0, double *sig,
                         uint64_t *seed_prefix);
int pgx_draw_pair_batch_gpu(PgxContext *ctx, int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c,
                            const int *ci, const int *n_clones, double dt_myr, int *clone_off, double *ps,
                            int *steps, double *dt, double *r50_pc, double *rtot_pc);
uint64_t pgx_seed_prefix(const char *target_id);

/* Pair jobs on the host (the reference's pair mode: phygas_cli's target loop, src/phygas_cli.c:37-51, and
 * ph_pair_draw, src/phygas.c:182-198):
 * pgx_prefilter_pairs -- the (target, cluster) pairs that pass ph_prefilter, tracks built as the reference's CLI
 *   builds them (32 spread clones, seeds ph_seed("track", id/name), traced back over the longest cluster tmax); pair
 *   k = (ti[k], ci[k]) in (target, cluster) order; at most cap pairs written, *n = how many pass.
 * pgx_draw_pair_batch -- ph_pair_draw for pair q = (t[ti[q]], c[ci[q]]) with its own clone count n_clones[q] and the
 *   pair's seed ph_seed(id, name): the clones of all pairs back to back in ps (room for 12 * sum(n_clones) doubles),
 *   clone_off[n_pairs + 1], and per pair steps, dt, r50_pc, rtot_pc -- the arguments of pgx_pair. */
/* The screen's chance-alignment control (reference src/phygas_screen.c:35-47): out[j] = t[j] with the proper motions
 * (rescaled by the parallax ratio) and the radial velocity of t[(j + n/2) % n]; out must not alias t. */
int pgx_control_targets(const PhTarget *t, int n, PhTarget *out);
int pgx_prefilter_pairs(const PhTarget *t, int nt, const PhCluster *c, int nc, int threads, int *ti, int *ci,
                        long cap, long *n);
int pgx_draw_pair_batch(int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c, const int *ci,
                        const int *n_clones, double dt_myr, int threads, int *clone_off, double *ps, int *steps,
                        double *dt, double *r50_pc, double *rtot_pc);
/* The prefilter on the GPU (reference ph_track_target / ph_track_cluster / ph_prefilter over every pair,
 * src/phygas.c:98-168, as src/phygas_cli.c:31-46 runs them): the same pairs in the same order as pgx_prefilter_pairs
 * (at most cap written to ti/ci, *n = how many pass).  The host draws the tracks' starts and spreads on `threads`
 * threads (0 = all cores); the GPU traces the coarse tracks and tests the pairs; the cluster tracks stay in the
 * context for the next call with the same clusters.  A pair the GPU cannot decide with the margin to spare is decided
 * by the host code.  Every cluster's tmax_myr must lie in [0, 1e5] (PGX_E_ARG otherwise).  pgx_stats: ms_prefilter
 * (device time), prefilter_pairs, prefilter_rechecked, body_steps. */
int pgx_prefilter(PgxContext *ctx, const PhTarget *t, int nt, const PhCluster *c, int nc, int threads, int *ti,
                  int *ci, long cap, long *n);
/* The distance (kpc, >= 0) the GPU's prefilter decisions keep from the threshold, a bound on how far a GPU-traced
 * track point may lie from the host-traced one (default 1e-7). */
int pgx_prefilter_margin(PgxContext *ctx, double margin_kpc);
/* Stage-2 pair selection (the reference BOINC app's pair mode, src/main_phygas_boinc.cpp:309-333 and 445-447): a
 * target whose lists[j] is a non-empty comma-separated list of cluster names ("clusters=" on its work-unit line)
 * runs exactly the clusters named there, in cluster order; every other target (lists NULL, or lists[j] NULL or "")
 * runs the clusters that pass the prefilter (pgx_prefilter).  Pairs in (target, cluster) order, at most cap written
 * to ti/ci, *n = how many. */
int pgx_pairs_with_lists(PgxContext *ctx, const PhTarget *t, int nt, const char *const *lists, const PhCluster *c,
                         int nc, int threads, int *ti, int *ci, long cap, long *n);
/* The clusters a "clusters=" list names (a name matches a whole comma-separated item): their indices, in cluster
 * order, at most cap written to ci; returns how many match. */
int pgx_cluster_list(const PhCluster *c, int nc, const char *list, int *ci, int cap);
/* Coarse tracks of n objects (reference track, src/phygas.c:98-111): from nominal starts ps (6 doubles each; kpc,
 * kpc/Myr), npts[i] points 0.5 Myr apart (10 KDK steps of -0.05 Myr): pos = 3 npts[i] doubles per object, back to
 * back. */
int pgx_tracks(PgxContext *ctx, int n, const double *ps, const int *npts, double *pos);

/* ---- pair Monte Carlo ------------------------------------------------------------------------------------------ */
/* Trace every clone of n_pairs pairs back and reduce each pair (reference ph_pair_clone + ph_pair_reduce,
 * src/phygas.c:200-238; GPU pg_pair + the host reduction of src/main_phygas_boinc.cpp:236-246).
 * Clones of pair p are clone_off[p] .. clone_off[p+1]-1 (clone_off[n_pairs] = total, at most 2^26 per pair);
 * ps = 12 doubles per clone as ph_pair_draw writes them; steps/dt per pair as ph_pair_draw returns them;
 * r50_pc/rtot_pc per pair.  res[n_pairs] gets the results; clone_out (NULL or 3 x total: best kpc, tbest Myr,
 * vbest kpc/Myr, clone-major blocks) the per-clone closest approaches. */
int pgx_pair(PgxContext *ctx, int n_pairs, const int *clone_off, const double *ps, const int *steps,
             const double *dt, const double *r50_pc, const double *rtot_pc, PhResult *res, double *clone_out);

/* Launch-shape autotuner of the clone kernel (no counterpart in the reference): runs the batch (the arguments of
 * pgx_pair) with every shape this build has -- warps per block x clones traced per lane x resident blocks per SM
 * asked of the compiler (a register cap) -- and keeps the fastest for
 * this context's later pgx_pair calls.  ms[pgx_pair_shapes()] (or NULL) gets each shape's device time; *best (or NULL)
 * its index.  Every shape must give the same bits: a shape whose results differ fails the call (PGX_E_CUDA).
 * Batches whose pairs all have at most 1024 clones run as one captured CUDA graph (prep, persistent trace, reduce)
 * replayed with the batch's parameters; the tuner's runs also capture each shape's graph. */
int pgx_tune_pair(PgxContext *ctx, int n_pairs, const int *clone_off, const double *ps, const int *steps,
                  const double *dt, const double *r50_pc, const double *rtot_pc, double *ms, int *best);
/* Launch-shape autotuner of the screen's block filter (no counterpart in the reference): screens the staged chunk
 * (pgx_screen_stage) with every shape of the filter -- resident blocks per SM asked of the compiler, which sets its
 * register cap -- and keeps the fastest for this context's later screens.  ms[pgx_screen_shapes(0, NULL)] (or NULL)
 * gets each shape's filter time (ms_scan), *best (or NULL) its index.  The shapes differ in register allocation only,
 * so they give the same rows; a shape that keeps another number of pairs fails the call (PGX_E_CUDA). */
int pgx_tune_screen(PgxContext *ctx, double tmax_myr, double chi2_max, double *ms, int *best);
/* number of the filter's launch shapes; the first n minimum resident blocks per SM into min_blocks */
int pgx_screen_shapes(int n, int *min_blocks);
/* number of launch shapes; the first n as (warps per block, clones per lane, minimum resident blocks per SM) */
int pgx_pair_shapes(int n, int *warps, int *clones_per_lane, int *min_blocks);
/* ph_pair over a list of (target, cluster) pairs -- pair q = (t[ti[q]], c[ci[q]]) with n_clones[q] clones, seeds
 * ph_seed(id, name), dt_myr as pgx_draw_pair_batch -- with the host draws pipelined: the clones of batch b + 1
 * (batch_pairs pairs; <= 0: 1,024) are drawn on `threads` host threads (<= 0: all cores) into page-locked memory
 * while the GPU traces batch b.  res[q] as pgx_pair gives it; pgx_stats sums the batches. */
int pgx_pair_targets(PgxContext *ctx, int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c, const int *ci,
                     const int *n_clones, double dt_myr, int threads, int batch_pairs, PhResult *res);
/* The persistent clone kernels of this context on at most blocks_per_sm blocks per SM (0 = as many as fit, the
 * default): leaves registers for other contexts' kernels to run beside them -- the request loop's slots. */
int pgx_pair_blocks(PgxContext *ctx, int blocks_per_sm);
/* The same cap, applied only to the launches made while *busy is nonzero (read atomically at each launch of a batch;
 * busy NULL: always, as pgx_pair_blocks): a caller that runs other work beside the clone kernels sets the flag
 * while that work runs, and the clone kernels take the whole GPU the rest of the time. */
int pgx_pair_blocks_while(PgxContext *ctx, int blocks_per_sm, const int *busy);

/* pgx_pair for callers that cannot allocate GPU memory (no counterpart in the reference): code running inside
 * another framework's device memory pool, loops that must not stall on the allocator, hosts that can only hand
 * over buffers they already own.  Every pointer is DEVICE memory the caller provides (clone_off[n_pairs + 1],
 * ps[12 * n_clones], steps/dt/r50_pc/rtot_pc[n_pairs], res[n_pairs]); n_clones = clone_off[n_pairs].  After the
 * first call on a device, a call only enqueues work on `stream` (a cudaStream_t, NULL = the legacy default stream)
 * of the current device and returns; res is complete when the stream reaches that point.  The first call on a
 * device does its set-up: it looks up the scratch array's address and fills the force tables with one kernel on the
 * legacy default stream, then synchronizes the whole device -- make it before any stream capture, at start-up.  No
 * cudaMalloc, cudaFree or allocating library call: the per-clone scratch is a fixed 24 MiB array inside the
 * library.  At most 2^20 clones per call (PGX_E_LIMIT beyond).  A pair gets n = -1 when it has more than 1024 clones
 * or when its offsets are not inside [0, n_clones] (a bad clone_off; the device offsets cannot be checked on the
 * host); a pair without clones gets the reference's zeroed result with n = 0.  The scratch is shared by all calls
 * and keeps the last call's contents: calls that overlap on the GPU race, so serialise them. */
int pgx_pair_noalloc(void *stream, int n_pairs, int n_clones, const int *clone_off, const double *ps,
                     const int *steps, const double *dt, const double *r50_pc, const double *rtot_pc, PhResult *res);

/* ---- measurement ------------------------------------------------------------------------------------------------ */
/* Device times (CUDA events on the context's stream) and counts of the last pgx_screen_exec / pgx_pair call. */
typedef struct {
    double ms_total, ms_orbit, ms_cov, ms_scan, ms_select, ms_finish, ms_pair;
    long pairs, kept, candidates, rechecked_points, rechecked_draws, clones, clone_steps, body_steps;
    long ambiguous;                  /* mixed screen: pairs that may be kept (candidates) whose candidate points
                                        were found by a second walk; rechecked_points = points evaluated in FP64 */
    int kernels;                     /* kernel launches of the call */
    long orbit_body_steps;           /* body steps of the orbit launch that ms_orbit times (a chunk screened in parts
                                        times the first part's; the others run beside the previous part's screen) */
    double ms_prefilter;             /* pgx_prefilter: device time of the tracks and the pair tests */
    long prefilter_pairs, prefilter_rechecked;   /* pairs tested; pairs within the margin, decided on the host */
    int parts;                       /* screen: the parts the chunk was screened in (1 = whole), one scan launch each */
} PgxStats;
int pgx_stats(const PgxContext *ctx, PgxStats *out);

/* Measured peak FMA rates of this GPU, in FLOP/s (2 per fused multiply-add): the roofline denominators of the
 * FP64-bound orbit stages and the FP32-bound filter.  Runs two short probe kernels (about 20 ms). */
int pgx_peaks(PgxContext *ctx, double *fp64_flops, double *fp32_flops);

/* Self-check of the mixed-precision screen's error bounds (no counterpart in the reference): for n points given in
 * FP64 -- pos[12n] = star and cluster positions at the point and at the next (t0 c0 t1 c1), S[12n] = the star's and
 * the cluster's covariance (xx xy xz yy yz zz), R2[n] -- returns the FP64 point chi2 (v64; -1 singular, +inf
 * rejected by the trace bound) and the FP32 filter's bounds lb <= v64 <= ub, or rej = 1 where the filter rejects
 * the point (then v64 >= chi2_max); rej = 2 where its cheap pre-test skips the point (then v64 >= chi2_max too; the
 * bounds are returned). */
int pgx_check_bounds(PgxContext *ctx, int n, const double *pos, const double *S, const double *R2, double chi2_max,
                     double *v64, float *lb, float *ub, int *rej);

/* Self-check of the mixed-precision filter's block test (no counterpart in the reference): on the chunk staged by
 * pgx_screen_stage (unsplit: pgx_screen_split(ctx, 0), or fewer stars than the split threshold), traces its tracks
 * (tmax_myr), runs the block test on every (pair, block of 8 points) as the filter does, and evaluates the FP64 point
 * chi2 of every point: counts[12] = blocks tested, blocks settled, points of settled blocks, violations (points of
 * settled blocks under chi2_max; 0 when the test's bounds hold), blocks whose points are all at or above chi2_max,
 * blocks of pairs with a point under it, points of the blocks not settled, of those the ones the filter's point test
 * settles, the ones at or above chi2_max, and the point tests' violations (0 when their bounds hold); then the ones
 * the point test against the block's dominating matrix settles, and of those the ones the point test leaves. */
int pgx_check_blocks(PgxContext *ctx, double tmax_myr, double chi2_max, long *counts);

/* Self-check of the mixed-precision finish's FP32 draws (no counterpart in the reference): for n pairs given by
 * fin11[11n] = (mx my mz, the covariance's Cholesky factor l00 l10 l20 l11 l21 l22, r50, rtot; kpc) and their draw
 * seeds, ratio[i] = the largest |x_j - x_j,64| / bound over the pair's 512 draws and three components, where x is
 * the FP32 draw, x_64 the FP64 path's and bound the FP32 draw's own error bound: <= 1 when the bound holds. */
int pgx_check_draws(PgxContext *ctx, int n, const double *fin11, const uint64_t *seed, double *ratio);

/* ---- serving ---------------------------------------------------------------------------------------------------- */
/* A request loop in front of the GPU (no counterpart in the reference, whose BOINC app runs one work unit at a time).
 * pgx_server_open creates `slots` device contexts, each with its own stream and its own resident copy of the cluster
 * table (clusters c, drawn once on the host with n_samp draws, kernel radius r_kernel as ph_screen_r).  Submitted
 * jobs queue in arrival order; a job starts when a slot is idle and the estimated device memory of the running jobs
 * plus its own stays within hbm_budget_gb (the first job of an idle GPU always starts).  Slots run their jobs' host
 * parts (draws, prefilter) on host_threads / slots cores (host_threads <= 0: all cores) while other slots' kernels run,
 * so jobs arriving while others are on the GPU are admitted as slots and memory free up and their work overlaps on the
 * device.  A job's results depend only on its inputs: the same bits alone and in any mix.
 * Kinds: PGX_JOB_SCREEN screens n_targets stars against the table (rows with p_r50 >= p_min kept, as the BOINC app's
 * emit cut); PGX_JOB_CONTROL the same on the velocity-shuffled chunk (pgx_control_targets); PGX_JOB_PAIRS runs the
 * pair Monte Carlo of n_targets targets against their prefiltered clusters (pgx_prefilter_pairs) with n_clones clones
 * at dt_myr.  Times are seconds since pgx_server_open; digest = FNV-1a 64 of the job's result records. */
#define PGX_JOB_SCREEN 0
#define PGX_JOB_CONTROL 1
#define PGX_JOB_PAIRS 2
typedef struct PgxServer PgxServer;
typedef struct {
    int kind;                 /* PGX_JOB_* */
    int precision;            /* screen and control: PGX_MIXED or PGX_FP64 */
    const PhTarget *targets;  /* copied by pgx_server_submit */
    int n_targets;
    double chi2_max;          /* screen and control */
    double p_min;             /* screen and control: keep rows with p_r50 >= p_min */
    int n_clones;             /* pairs */
    double dt_myr;            /* pairs */
} PgxJob;
typedef struct {
    int status;               /* PGX_OK or the job's error code (-1 while it runs) */
    int kind, slot;
    double t_submit, t_start, t_end;
    long n_out;               /* screen rows kept, or pairs traced */
    double work;              /* star-cluster pairs screened, or clone-steps */
    uint64_t digest;
} PgxJobResult;
typedef struct {
    long submitted, finished, queued;
    int running, max_running, slots;
    double hbm_budget_gb, hbm_in_use_gb, hbm_peak_gb, now_s;
} PgxServerStats;
int pgx_server_open(int device, int slots, double hbm_budget_gb, const PhCluster *c, int nc, int n_samp,
                    double r_kernel, int host_threads, PgxServer **out);
int pgx_server_submit(PgxServer *s, const PgxJob *job, long *id);
int pgx_server_wait(PgxServer *s, long id, PgxJobResult *out);     /* blocks until the job has finished */
/* the same for at most timeout_s seconds: PGX_E_TIMEOUT (out = the job's state so far) when it has not finished */
int pgx_server_wait_for(PgxServer *s, long id, double timeout_s, PgxJobResult *out);
int pgx_server_query(PgxServer *s, long id, PgxJobResult *out);    /* PGX_E_PENDING until then */
/* a finished job's results (cap records at most; returns the count, -1 if unknown or unfinished):
 * screen and control rows, or the pair jobs' PhResult with each pair's cluster index */
long pgx_server_rows(PgxServer *s, long id, PgxScreenRow *rows, long cap);
long pgx_server_pairs(PgxServer *s, long id, PhResult *res, int *cluster, long cap);
void pgx_server_release(PgxServer *s, long id);                    /* forget a finished job */
int pgx_server_stats(PgxServer *s, PgxServerStats *out);
void pgx_server_close(PgxServer *s);                               /* finishes the queued jobs first */

#ifdef __cplusplus
}
#endif
#endif
