// pgx_scan.cu -- the star x cluster screen of libphygas_gb300 in FP64, and the stages every screen path shares.
//
// Built with --fmad=false: the per-point chi2 (reference ph_screen_chi2_cut, src/phygas.c:370-407) and the
// 512-draw probabilities (reference ph_screen_finish, src/phygas.c:413-444) are evaluated with the reference's
// operation order and no contraction, so that on identical tracks they give the reference's bits, and so that the
// FP64 path and the FP64 rechecks of the mixed-precision path (pgx_mixed.cu, which includes the same functions)
// can never disagree.
//
//   k_scan64       one thread per (star, cluster) pair: warp = 32 stars x one cluster (same track length, the
//                  cluster's points are a broadcast load); writes chi2, kb, sb per pair, cluster-major
//   k_count_kept / k_exclusive_scan / k_emit_kept   stable compaction of the pairs under the cut, (star, cluster)
//   k_finish_prep  one thread per kept pair: interpolated separation, speeds, sigma, Cholesky factor, pair seed
//   k_finish64     one warp per kept pair: its 512 draws x 3 Gaussians in FP64 (lane = 16 draws), counts by shuffle
#include "pgx_internal.cuh"
#include "pgx_kernels.h"
#include "pgx_screen_math.cuh"

namespace pgx {

__global__ void __launch_bounds__(128) k_scan64(ScreenTables T, double cut, double *__restrict__ chi2T,
                                                int *__restrict__ kbT, double *__restrict__ sbT) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= T.nt) return;
    const size_t NT = T.nt, NC = T.nc;
    for (int c = blockIdx.y; c < T.nc; c += gridDim.y) {
        const int n = T.ns < T.cn[c] ? T.ns : T.cn[c];
        ScanState st;
        st.begin();
        const double R2 = T.R2[c];
        for (int k = 0; k < n; k++) {
            const double *tk = T.t64 + (size_t)k * 12 * NT + s, *ck = T.c64 + (size_t)k * 12 * NC + c;
            double M[6], m0[3], m1[3];
#pragma unroll
            for (int i = 0; i < 6; i++) M[i] = tk[(6 + i) * NT] + __ldg(ck + (6 + i) * NC);
#pragma unroll
            for (int i = 0; i < 3; i++) m0[i] = tk[i * NT] - __ldg(ck + i * NC);
            const bool more = k + 1 < n;
            if (more) {
                const double *tn = tk + 12 * NT, *cm = ck + 12 * NC;
#pragma unroll
                for (int i = 0; i < 3; i++) m1[i] = tn[i * NT] - __ldg(cm + i * NC);
            } else {
                m1[0] = m0[0]; m1[1] = m0[1]; m1[2] = m0[2];
            }
            st.point(k, M, R2, m0, m1, more, cut);
        }
        const size_t o = (size_t)c * NT + s;
        chi2T[o] = st.best;
        kbT[o] = st.kb;
        sbT[o] = st.sb;
    }
}

__global__ void k_count_kept(int nt, int nc, const double *__restrict__ chi2T, double cut, int *__restrict__ cnt) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nt) return;
    int n = 0;
    for (int c = 0; c < nc; c++) n += chi2T[(size_t)c * nt + s] < cut;
    cnt[s] = n;
}

// exclusive prefix sum of n ints by one CTA of 1024 threads (n is a star count: a few 10^4)
__global__ void __launch_bounds__(1024) k_exclusive_scan(int n, const int *__restrict__ in, int *__restrict__ out,
                                                         int *__restrict__ total) {
    __shared__ int part[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < n ? in[i] : 0;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int d = 1; d < 1024; d <<= 1) {
            const int add = threadIdx.x >= d ? part[threadIdx.x - d] : 0;
            __syncthreads();
            part[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < n) out[i] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += part[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_emit_kept(int nt, int nc, const double *__restrict__ chi2T, const int *__restrict__ kbT,
                            const double *__restrict__ sbT, double cut, const int *__restrict__ off,
                            KeptPair *__restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nt) return;
    int j = off[s];
    for (int c = 0; c < nc; c++) {
        const size_t o = (size_t)c * nt + s;
        const double q = chi2T[o];
        if (q < cut) {
            KeptPair p;
            p.s = s; p.c = c; p.kb = kbT[o]; p.pad = 0; p.sb = sbT[o]; p.chi2 = q;
            out[j++] = p;
        }
    }
}

__global__ void k_finish_prep(ScreenTables T, int n, const KeptPair *__restrict__ kp, FinishIn *__restrict__ fin,
                              ScreenRowDev *__restrict__ rows) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= n) return;
    const KeptPair p = kp[h];
    FinishIn f;
    ScreenRowDev r;
    finish_prep_pair(T, p, f, r);
    fin[h] = f;
    rows[h] = r;
}

__global__ void __launch_bounds__(256) k_finish64(int n, const FinishIn *__restrict__ fin,
                                                  ScreenRowDev *__restrict__ rows) {
    const int h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (h >= n) return;
    const FinishIn f = fin[h];
    int in50 = 0, intot = 0;
#pragma unroll 1
    for (int q = 0; q < 16; q++) {
        const int i = lane + 32 * q;
        const int v = draw_inside64(f, i);
        in50 += v & 1;
        intot += v >> 1;
    }
    in50 = __reduce_add_sync(0xffffffffu, in50);
    intot = __reduce_add_sync(0xffffffffu, intot);
    if (lane == 0) {
        rows[h].p_r50 = (double)in50 / 512.0;
        rows[h].p_rtot = (double)intot / 512.0;
    }
}

}  // namespace pgx
