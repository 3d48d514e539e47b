// pgx_mixed.h -- the mixed-precision screen stages and the cluster-table helpers (internal header).
#pragma once
#include <string>
#include "pgx_kernels.h"
#include "phygas_gb300.h"

namespace pgx {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

// work buffers of the mixed-precision screen, owned by the context
struct MixedBufs {
    DevBuf order, ub, kmin, flag, cnt, off, total, kept, cand, cand_off, ent, entq, aux, ovf;
    std::string err;
    int scan_variant = 0;             // the block filter's launch shape (scan_shape), chosen by the screen autotuner
};
// the block filter's launch shapes: how many, and shape v's resident blocks per SM asked of the compiler
int scan_shapes();
int scan_shape(int v);

void mixed_free(MixedBufs &m);
// a device buffer of at least `bytes` (grown by a quarter more when it has to grow); a CUDA status as a PGX code
int grow(DevBuf &b, size_t bytes, std::string &err);
int check(cudaError_t e, std::string &err, const char *what);
// exclusive scan of n ints into out, the total into *total (device); part: n / 1024 + 2 ints of scratch
int exclusive_scan(cudaStream_t st, int n, const int *in, int *out, int *part, int *total, std::string &err);
// slot-ordered tracks (longest first) -> cluster-ordered table columns
int gather_columns(cudaStream_t st, int nc, int nmax, const int *order_host, const double *t64_slot,
                   const float4 *t32_slot, const float *lm_slot, double *c64, float4 *c32, float *clm, MixedBufs &m);
// the kernel radius folded into the FP32 cluster table the filter reads: S + R^2 I and lmin + R^2 (once per table)
int mixed_cluster_aux(cudaStream_t st, int nc, int nmax, const int *cn, const double *c64, const double *R2,
                      float4 *c32, float *clm, MixedBufs &m);
// the block tables of N objects' tracks (t64 [k][12][N], lm [k][N], npts[i] points or nmax for all, R2[i] on S's
// diagonal or none) into blk [ceil(nmax / kBlk)][N][4] float4: what the filter's block test reads
int block_tables(cudaStream_t st, int N, int nmax, const int *npts, const double *t64, const float *lm,
                 const double *R2, float4 *blk, std::string &err);
// the draws from the measurement errors on the device (pgx_draws.cu): targets' and clusters' nominal states and
// covariances (seed[i] = ph_seed("lin", id)), and the clones of pairs (seed[q] = ph_seed(id, name), clone slots
// slot[q], successful clones m[q]); every pointer is device memory
int draw_targets_gpu(cudaStream_t st, int n, const PhTarget *t, int n_samp, const uint64_t *seed, double *ps0,
                     double *sig, std::string &err);
int draw_clusters_gpu(cudaStream_t st, int n, const PhCluster *c, int n_samp, const uint64_t *seed, double *ps0,
                      double *sig, std::string &err);
int draw_pairs_gpu(cudaStream_t st, int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c,
                   const int *ci, const int *n_clones, const uint64_t *seed, const long long *slot, double *ps,
                   int *m, std::string &err);
int compact_pairs_gpu(cudaStream_t st, int n_pairs, const long long *slot, const int *off, const int *m,
                      const double *src, double *dst, std::string &err);
// the cluster table cluster-major (blk [nblk][nc][4] -> [nc][nblk][4], c32 [ncp][nc][3] -> [nc][ncp][3], lm
// [ncp][nc] -> [nc][lm_pitch]): the staged filter's bulk copies read contiguous ranges
int cluster_major(cudaStream_t st, int nc, int ncp, int nblk, int lm_pitch, const float4 *blk, const float4 *c32,
                  const float *lm, float4 *blk_cm, float4 *c32_cm, float *lm_cm, std::string &err);
// FP32 filter + FP64 recheck: the kept pairs in (star, cluster) order, identical to the FP64 path's
int mixed_select(cudaStream_t st, const ScreenTables &T, double cut, MixedBufs &m, cudaEvent_t ev_scan, int *total,
                 PgxStats *stats);
const KeptPair *mixed_kept(MixedBufs &m);
// FP32 draws with an FP64 guard band: counts identical to the FP64 path's
int mixed_finish(cudaStream_t st, int n, const FinishIn *fin, ScreenRowDev *rows, MixedBufs &m, PgxStats *stats);

// self-check of the FP32 point bounds (pgx_check_bounds)
// self-check of the FP32 draws' error bound (pgx_check_draws)
int mixed_check_draws(cudaStream_t st, int n, const FinishIn *fin, double *ratio, std::string &err);
int mixed_check_bounds(cudaStream_t st, int n, const double *pos, const double *S, const double *R2, double cut,
                       double *v64, float *lb, float *ub, int *rej, std::string &err);
// self-check of the filter's block test on the staged chunk's tracks (pgx_check_blocks): cnt[4] on the device
// counters of pgx_check_blocks
constexpr int kCheckBlockCounts = 12;
int mixed_check_blocks(cudaStream_t st, const ScreenTables &T, double cut, unsigned long long *cnt, std::string &err);

}  // namespace pgx
