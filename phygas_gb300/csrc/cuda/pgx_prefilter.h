// pgx_prefilter.h -- the pair prefilter on the GPU (internal header).
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include "pgx_mixed.h"
#include "phygas.h"

namespace pgx {

// kpc: the margin the GPU's decisions keep from the prefilter's threshold.  It bounds the distance between a coarse
// track point traced on the GPU and the same point traced by the host code (the force's last bits differ, as any two
// libms' do; the tests find them within 1e-11 kpc on 100 Myr tracks).  Pairs inside the margin are decided on the host.
constexpr double kPrefilterMargin = 1e-7;

struct PrefilterState {
    // the cluster side, kept while the same clusters come back: nominal starts, spreads, points, r0 and the tracks
    DevBuf c_ps, c_sig, c_n, c_r0, c_pos;
    uint64_t digest = 0;
    int nc = 0;
    std::vector<PhTrack> host_ctr;           // host-traced cluster tracks for the rechecks (n = 0: not traced yet)
    // per call
    DevBuf t_ps, t_sig, t_n, t_pos, keep;
    std::vector<unsigned char> h_keep;
    double margin = kPrefilterMargin;
};

struct PrefilterCounts {
    long pairs = 0, rechecked = 0, body_steps = 0;
    int kernels = 0;
    float ms_device = 0.f;                   // the call's launches, CUDA events on the stream
};

// the (target, cluster) pairs of t[0, nt) x c[0, nc) that pass ph_prefilter (tracks as the reference's pair CLI
// builds them: 32 spread draws, seeds ph_seed("track", id/name), targets traced over the longest cluster tmax), in
// (target, cluster) order: at most cap written to ti/ci, *n = how many pass.  The same pairs as the host's
// pgh_prefilter_pairs: pairs the GPU cannot decide with the margin to spare are decided by the host code.
int prefilter_pairs(cudaStream_t st, PrefilterState &P, const PhTarget *t, int nt, const PhCluster *c, int nc,
                    int threads, int *ti, int *ci, long cap, long *n, PrefilterCounts &cnt, std::string &err);
// coarse tracks of n objects from their nominal starts (6 doubles each): pos = 3 npts[i] doubles per object, back to
// back in object order
int coarse_tracks(cudaStream_t st, PrefilterState &P, int n, const double *ps, const int *npts, double *pos,
                  std::string &err);
void prefilter_free(PrefilterState &P);

}  // namespace pgx
