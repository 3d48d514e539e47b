// pgx_kernels.h -- kernels of libphygas_gb300 and the device-side argument records they take (internal header).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pgx {

// layout-identical to PhResult (include/phygas.h); checked by a static_assert in pgx_api.cu
struct PhResultDev {
    int n, pad;          // pad: PhResult's alignment gap, written as 0 so the results are fully defined bytes
    double d05, d50, d95, t05, t50, t95, v05, v50, v95, f_r50, f_rtot;
};

constexpr int kMcThreads = 128;

// Clone Monte Carlo work: clones of pair p are [clone_off[p], clone_off[p+1]); ps = 12 doubles per clone
struct McPairs {
    int n_pairs, n_clones, n_items;
    const int *clone_off;     // n_pairs + 1
    const double *ps;         // n_clones * 12
    const int *steps;         // per pair
    const double *dt;         // per pair (negative)
    const double *r50_pc, *rtot_pc;
    const int4 *items;        // (pair, first clone, count <= 32, -)
    int *qhead;               // queue head (zeroed before launch)
    int *done;                // per pair, clones finished (zeroed before launch)
    double *cres;             // [3][n_clones]: best (kpc), tbest (Myr), vbest (kpc/Myr)
    PhResultDev *res;         // per pair
};

// points per block of the mixed filter's block test (pgx_bounds32.cuh kBlk)
constexpr int kBlockPoints = 8;

// The screen's device tables.  Star tracks: FP64 t64[k][12][nt] (pos, vel, S) and FP32 t32[k][nt][3] float4
// (pos hi, pos lo, S).  Cluster table: the same two layouts over nc, plus per cluster its point count, kernel
// radius^2, r50 and rtot (kpc) and its name (for the pair seeds).
struct ScreenTables {
    int nt, ns;                      // stars, points per star track
    int nc, ncp;                     // clusters, points of the longest cluster track
    const double *t64;
    const float4 *t32;
    const float *lm_t;               // [k][nt]: lower bound on lambda_min(S) of the star track (FP32, rounded down)
    const uint64_t *seed_prefix;     // per star: FNV-1a state after "id|"
    const double *c64;
    const float4 *c32;               // the cluster table in FP32 with the kernel radius folded in: S + R^2 I
    const float *lm_c;               // [k][nc]: lower bound on lambda_min(S) + R^2 (FP32, rounded down)
    // per object and block of kBlockPoints points, the block test's data ([b][n][4] float4, pgx_bounds32.cuh
    // block_skip32); nullptr: the mixed filter walks every point
    const float4 *blk_t = nullptr, *blk_c = nullptr;
    // the cluster table cluster-major, for the filter variant that copies a cluster's data into shared memory with
    // bulk copies (TMA): blk_cm [nc][nblk][4], c32_cm [nc][ncp][3] float4, lm_cm [nc][lm_pitch] (nullptr: not staged);
    // wait_err: set when a bulk copy's wait ran out (never expected; the host reports it)
    const float4 *blk_cm = nullptr, *c32_cm = nullptr;
    const float *lm_cm = nullptr;
    int nblk = 0, lm_pitch = 0;
    int *wait_err = nullptr;
    const int *cn;
    const double *R2, *r50, *rtot;
    const char *cname;               // nc * 40 bytes
    int s_off;                       // added to the star index of the rows written (a chunk screened in parts)
};

// one pair kept past the chi2 cut, in (star, cluster) order
struct KeptPair {
    int s, c, kb, pad;
    double sb, chi2;
};

// what the 512-draw stage needs of a kept pair, and the row it fills
struct FinishIn {
    double mx, my, mz, l00, l10, l20, l11, l21, l22, r50, rt;
    uint64_t seed;
};
struct ScreenRowDev {                // layout-identical to PgxScreenRow (include/phygas_gb300.h)
    int star, cluster, kb, pad;
    double sb, chi2, t_myr, d_nom_pc, sig_pc, p_r50, p_rtot, vrel_kms;
};

// the orbit force's tables, filled once per device (0 ok); before any orbit kernel, outside stream capture
int orbit_setup(int dev);

// ---- kernels ------------------------------------------------------------------------------------------------------
__global__ void k_stm_orbits(int N, const double *ps0, const int *npts, int nmax, double *opos, double *ovel);
__global__ void k_stm_cov(int N, int nmax, const int *npts, const double *opos, const double *ovel,
                          const double *sig21, double *t64, float4 *t32, float *lm);
// the prefilter's coarse tracks: nominal orbits from ps (6 doubles per object), pos[k][3][N] for k < npts[i]
cudaError_t launch_coarse_tracks(cudaStream_t st, int N, const double *ps, const int *npts, double *pos);
__global__ void k_pair_mc(McPairs P);
// launch-shape variants of the persistent clone kernel (parameters in device memory): count, shape (warps per block,
// clones per lane), full persistent grid, and the prep + trace + reduce kernels as one sequence on a stream (pairs of
// at most 1024 clones)
int mc_variants();
void mc_variant_shape(int v, int &warps, int &cpl, int &min_blocks);
cudaError_t mc_variant_grid(int v, int sms, int &grid);
cudaError_t launch_mc(int v, int grid, int prep_grid, int reduce_grid, cudaStream_t st, const McPairs *Pd);
// pairs of more than 1024 clones: sorted in shared memory up to kSortMax clones (dynamic shared memory of the launch:
// the batch's largest such pair rounded up to a power of two, times 8 bytes), beyond that reduced by radix selection
constexpr int kSortMax = 16384;
// the most clones of one pair (the clone offsets are 32-bit)
constexpr int kMaxPairClones = 1 << 26;
__global__ void k_pair_reduce_big(McPairs P);
__global__ void k_pair_reduce_only(McPairs P);
__global__ void k_peak_dfma(double *out, int iters, double a, double b);
__global__ void k_peak_ffma(float *out, int iters, float a, float b);

__global__ void k_scan64(ScreenTables T, double cut, double *chi2T, int *kbT, double *sbT);
__global__ void k_count_kept(int nt, int nc, const double *chi2T, double cut, int *cnt);
__global__ void k_exclusive_scan(int n, const int *in, int *out, int *total);
__global__ void k_emit_kept(int nt, int nc, const double *chi2T, const int *kbT, const double *sbT, double cut,
                            const int *off, KeptPair *out);
__global__ void k_finish_prep(ScreenTables T, int n, const KeptPair *kp, FinishIn *fin, ScreenRowDev *rows);
__global__ void k_finish64(int n, const FinishIn *fin, ScreenRowDev *rows);

}  // namespace pgx
