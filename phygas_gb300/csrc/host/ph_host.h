/* ph_host.h -- internal host helpers of libphygas_gb300 (not part of the public C-ABI). */
#ifndef PH_HOST_H
#define PH_HOST_H
#include <stdint.h>
#include <unistd.h>
#include "phygas.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ph_lin_target_init / the cluster counterpart with the covariance as 36 doubles, row-major */
void pgh_target_init(const PhTarget *t, int n_samp, uint64_t seed, double ps0[6], double sig[36]);
void pgh_cluster_init(const PhCluster *c, int n_samp, uint64_t seed, double ps0[6], double sig[36]);
/* the same for n objects on `threads` host threads (seeds ph_seed("lin", id|name)); prefix may be NULL */
void pgh_draw_targets(const PhTarget *t, int n, int n_samp, int threads, double *ps0, double *sig, uint64_t *prefix);
void pgh_draw_clusters(const PhCluster *c, int n, int n_samp, int threads, double *ps0, double *sig);
/* FNV-1a: state after "target_id|", and its continuation over a string (ph_seed = continue(prefix(a), b)) */
uint64_t pgh_seed_prefix(const char *target_id);
uint64_t pgh_fnv_continue(uint64_t h, const char *s);
int pgh_default_threads(void);
/* fn(arg, i0, i1) over [0, n) in chunks, on `threads` host threads */
void pgh_parallel_for(int n, int threads, int chunk, void (*fn)(void *, int, int), void *arg);
/* ph_pair_draw for n_pairs pairs (clones of pair i at ps + 12 * n_clones * i; m, steps, dt per pair) */
void pgh_draw_pairs(int n_pairs, const PhTarget *const *t, const PhCluster *const *c, int n_clones, double dt_myr,
                    const uint64_t *seed, int threads, double *ps, int *m, int *steps, double *dt);
/* pairs (ti[k], ci[k]) of targets x clusters that pass ph_prefilter (tracks as phygas_cli builds them), in (target,
 * cluster) order; writes at most cap pairs and returns how many pass (-1: out of memory) */
long pgh_prefilter_pairs(const PhTarget *t, int nt, const PhCluster *c, int nc, int threads, int *ti, int *ci,
                         long cap);
/* the start of each coarse track as ph_track_target / ph_track_cluster build it (32 spread draws, seeds
 * ph_seed("track", id/name)), without the track: of n targets (t != NULL) or n clusters, on `threads` host threads;
 * ps = the nominal phase-space point (6 doubles per object), sig = (sig_pos, sig_vel) per object */
void pgh_track_starts(const PhTarget *t, const PhCluster *c, int n, int threads, double *ps, double *sig);
/* ph_pair_draw for pair q = (t[ti[q]], c[ci[q]]) with n_clones[q] clones, seeds ph_seed(id, name); the clones of all
 * pairs written back to back into ps (room for 12 * sum(n_clones) doubles) with clone_off[n_pairs + 1]; steps, dt,
 * r50_pc, rtot_pc per pair.  Returns 0, or -1 (out of memory), -2 (more than 2^31 - 1 clones) */
/* the screen's chance-alignment control: velocities of the star n/2 further on, proper motions rescaled by the
 * parallax ratio (out may not alias t) */
void pgh_control_targets(const PhTarget *t, int n, PhTarget *out);
int pgh_draw_pair_batch(int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c, const int *ci,
                        const int *n_clones, double dt_myr, int threads, int *clone_off, double *ps, int *steps,
                        double *dt, double *r50_pc, double *rtot_pc);

#ifdef __cplusplus
}
#endif
#endif
