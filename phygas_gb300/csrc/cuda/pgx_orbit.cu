// pgx_orbit.cu -- FP64 orbit kernels of libphygas_gb300: the state-transition tracks of the linear screen and the
// clone Monte Carlo of ph_pair with its quantile reduction.
//
//   k_stm_orbits   one thread per orbit: an object's nominal orbit and its 6 neighbours (+1e-5 on one phase-space
//                  axis) are 7 independent threads, so a warp is 32 orbits with identical work and no barrier
//                  (reference lin_integrate, src/phygas.c:286-323)
//   k_stm_cov      one thread per (object, point): A = (neighbour - nominal) / eps, S = A Sigma0 A^T, and the
//                  track layouts the screen reads (FP64 for the exact stages, split FP32 for the filter, and a
//                  lower bound on the smallest eigenvalue of S for the filter's error bounds)
//   k_pair_mc      persistent: warps take items of <= 32 clones of one pair from a device queue (longest first),
//                  trace them back with KDK leapfrog and the segment closest approach (reference ph_pair_clone,
//                  src/phygas.c:200-216); the warp that finishes a pair's last item reduces it in registers
//                  with warp shuffles (reference ph_pair_reduce, src/phygas.c:218-238)
//   k_pair_reduce_big  the same reduction for pairs of more than 1024 clones, one CTA per pair in shared memory
//   k_mc_prep, k_pair_mc_t, k_pair_reduce_dev  the same work as one captured CUDA graph for batches of pairs of at
//                  most 1024 clones: parameters read from device memory, tracing separate from the reduction, and
//                  the tracing kernel's launch shape (warps per block, clones per lane) a template the autotuner picks
//
// Built with --fmad=false: every fused multiply-add is an explicit fma(), so the rounding does not depend on how the
// compiler arranges a kernel, and every launch shape gives the same bits.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "phygas_gb300.h"
#include "pgx_force.cuh"
#include "pgx_kernels.h"

namespace pgx {

// npts == nullptr: every object has nmax points.  Orbit t of the 7 N (object i = t % N, axis j = t / N) per
// thread, grid-stride, so a small grid can trace a chunk beside other work (one orbit per thread with a full grid).
__global__ void __launch_bounds__(128) k_stm_orbits(int N, const double *__restrict__ ps0, const int *__restrict__ npts,
                                                    int nmax, double *__restrict__ opos, double *__restrict__ ovel) {
    const size_t NN = N;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < 7 * NN; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % NN), j = (int)(t / NN);
        Orbit o;
        o.x = ps0[i]; o.y = ps0[NN + i]; o.z = ps0[2 * NN + i];
        o.vx = ps0[3 * NN + i]; o.vy = ps0[4 * NN + i]; o.vz = ps0[5 * NN + i];
        switch (j) {
            case 1: o.x += kEps; break;
            case 2: o.y += kEps; break;
            case 3: o.z += kEps; break;
            case 4: o.vx += kEps; break;
            case 5: o.vy += kEps; break;
            case 6: o.vz += kEps; break;
            default: break;
        }
        o.init();
        const int n = npts ? npts[i] : nmax;
        constexpr double dt = -kStepMyr / kSub, h = 0.5 * dt;
        for (int k = 0; k < n; k++) {
            if (k > 0) {
#pragma unroll 1
                for (int s = 0; s < kSub; s++) o.kdk(dt, h);
            }
            double *p = opos + (size_t)(k * 7 + j) * 3 * NN + i;
            p[0] = o.x; p[NN] = o.y; p[2 * NN] = o.z;
            if (j == 0) {
                double *v = ovel + (size_t)k * 3 * NN + i;
                v[0] = o.vx; v[NN] = o.vy; v[2 * NN] = o.vz;
            }
        }
    }
}

// Coarse tracks of the prefilter (reference track, src/phygas.c:98-111): the nominal orbit of each object from ps
// (6 doubles per object), one thread per object; pos[k][3][N] = the position after 10 k KDK steps of -0.05 Myr, for
// k < npts[i].  The same orbit, steps and force as k_stm_orbits' nominal orbit.
__global__ void __launch_bounds__(32) k_coarse_tracks(int N, const double *__restrict__ ps,
                                                      const int *__restrict__ npts, double *__restrict__ pos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const size_t NN = N;
    const double *q = ps + 6 * (size_t)i;
    Orbit o;
    o.x = q[0]; o.y = q[1]; o.z = q[2]; o.vx = q[3]; o.vy = q[4]; o.vz = q[5];
    o.init();
    const int n = npts[i];
    constexpr double dt = -kStepMyr / kSub, h = 0.5 * dt;
    for (int k = 0; k < n; k++) {
        if (k > 0) {
#pragma unroll 1
            for (int s = 0; s < kSub; s++) o.kdk(dt, h);
        }
        double *p = pos + (size_t)k * 3 * NN + i;
        p[0] = o.x; p[NN] = o.y; p[2 * NN] = o.z;
    }
}

cudaError_t launch_coarse_tracks(cudaStream_t st, int N, const double *ps, const int *npts, double *pos) {
    if (N <= 0) return cudaSuccess;
    // a warp per block: the few hundred to few thousand orbits spread over every SM, each warp with an SM's FP64
    // pipe to itself
    k_coarse_tracks<<<(N + 31) / 32, 32, 0, st>>>(N, ps, npts, pos);
    return cudaGetLastError();
}

// sig21: the 21 distinct entries of the symmetric 6x6 Sigma0, [21][N], upper triangle row by row
__global__ void __launch_bounds__(256) k_stm_cov(int N, int nmax, const int *__restrict__ npts,
                                                 const double *__restrict__ opos, const double *__restrict__ ovel,
                                                 const double *__restrict__ sig21, double *__restrict__ t64,
                                                 float4 *__restrict__ t32, float *__restrict__ lm) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t NN = N;
    if (idx >= NN * nmax) return;
    const int i = (int)(idx % NN), k = (int)(idx / NN);
    if (npts && k >= npts[i]) return;
    const double *P = opos + (size_t)k * 21 * NN + i;
    const double x0 = P[0], y0 = P[NN], z0 = P[2 * NN];
    double A[3][6];
#pragma unroll
    for (int j = 0; j < 6; j++) {
        const double *Q = P + (size_t)(j + 1) * 3 * NN;
        A[0][j] = (Q[0] - x0) * 1e5;
        A[1][j] = (Q[NN] - y0) * 1e5;
        A[2][j] = (Q[2 * NN] - z0) * 1e5;
    }
    double sg[6][6];
    {
        int q = 0;
#pragma unroll
        for (int a = 0; a < 6; a++)
#pragma unroll
            for (int b = a; b < 6; b++) { sg[a][b] = sg[b][a] = sig21[(size_t)q * NN + i]; q++; }
    }
    double AS[3][6];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int b = 0; b < 6; b++) {
            double acc = 0.0;
#pragma unroll
            for (int a = 0; a < 6; a++) acc = fma(A[r][a], sg[a][b], acc);
            AS[r][b] = acc;
        }
    double S[6];
    const int rr[6] = {0, 0, 0, 1, 1, 2}, ss[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int q = 0; q < 6; q++) {
        double acc = 0.0;
#pragma unroll
        for (int b = 0; b < 6; b++) acc = fma(AS[rr[q]][b], A[ss[q]][b], acc);
        S[q] = acc;
    }
    const double *V = ovel + (size_t)k * 3 * NN + i;
    double *T = t64 + (size_t)k * 12 * NN + i;
    const double vals[12] = {x0, y0, z0, V[0], V[NN], V[2 * NN], S[0], S[1], S[2], S[3], S[4], S[5]};
#pragma unroll
    for (int f = 0; f < 12; f++) T[(size_t)f * NN] = vals[f];
    const float hx = (float)x0, hy = (float)y0, hz = (float)z0;
    float4 *o = t32 + ((size_t)k * NN + i) * 3;
    o[0] = make_float4(hx, hy, hz, (float)(x0 - (double)hx));
    o[1] = make_float4((float)(y0 - (double)hy), (float)(z0 - (double)hz), (float)S[0], (float)S[1]);
    o[2] = make_float4((float)S[2], (float)S[3], (float)S[4], (float)S[5]);
    // lower bound on lambda_min(S), rounded down to FP32, for the mixed-precision filter's error bounds
    const double l = sym3_min_eig_lb(S[0], S[1], S[2], S[3], S[4], S[5]);
    lm[(size_t)k * NN + i] = __double2float_rd(l - 1e-12 * fabs(l));
}

// ---------------------------------------------------------------------------------------------------------------
// clone Monte Carlo

// |v| in FP32 (components already in FP32), bounded from below (lo) or above (hi): the approximate square root is
// within a few ulp, and the 1e-6 margins cover it; outside 1e-18 <= |v| <= 1e18 the bounds are 0 and +inf
__device__ __forceinline__ float norm32_rsqrt(float q) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(q));
    return r;
}
__device__ __forceinline__ float norm32_lo(float x, float y, float z) {
    const float q = fmaf(x, x, fmaf(y, y, z * z));
    return q >= 1e-36f && q <= 1e36f ? q * norm32_rsqrt(q) * (1.f - 1e-6f) : 0.f;
}
__device__ __forceinline__ float norm32_hi(float x, float y, float z) {
    const float q = fmaf(x, x, fmaf(y, y, z * z));
    return q >= 1e-36f && q <= 1e36f ? q * norm32_rsqrt(q) * (1.f + 1e-6f) : __int_as_float(0x7f800000);
}

// One clone traced back: the target's and the cluster's orbit, the closest approach so far (reference
// ph_pair_clone and seg_min, src/phygas.c:147-156, 200-216).  Results in kpc, Myr, kpc/Myr.
//
// Each step's segment r0 -> r1 first gets an FP32 lower bound on its distance from the origin: every point of it is
// within |r1 - r0| / 2 of r0 or of r1, so none is nearer than min(|r0|, |r1|) - |r1 - r0| / 2.  The separations in
// FP32 are truncated (never above |r|) and the FP32 norms carry 1e-6 margins; when the bound exceeds the closest
// approach so far (an upper bound of it in FP32, with an absolute margin for the FP64 path's own rounding), the
// segment cannot improve it and the FP64 segment test is skipped.  Otherwise the reference's test runs as before,
// so the results are the same bits -- and the FP64 pipe does that work only near the closest approach.
struct Clone {
    Orbit a, b;
    double r0x, r0y, r0z, best, tbest, vbest;
    float f0x, f0y, f0z, n0, best_up;          // r0 truncated to FP32, |r0| from below, best from above
    __device__ __forceinline__ void set_best_up() { best_up = fmaf(f32_trunc(best), 1.f + 2.4e-7f, 1e-37f); }
    __device__ __forceinline__ void start(const double *__restrict__ ps) {
        a.x = ps[0]; a.y = ps[1]; a.z = ps[2]; a.vx = ps[3]; a.vy = ps[4]; a.vz = ps[5];
        b.x = ps[6]; b.y = ps[7]; b.z = ps[8]; b.vx = ps[9]; b.vy = ps[10]; b.vz = ps[11];
        a.init();
        b.init();
        r0x = a.x - b.x; r0y = a.y - b.y; r0z = a.z - b.z;
        best = sqrt(fma(r0x, r0x, fma(r0y, r0y, r0z * r0z)));
        tbest = 0.0;
        const double ux = a.vx - b.vx, uy = a.vy - b.vy, uz = a.vz - b.vz;
        vbest = sqrt(fma(ux, ux, fma(uy, uy, uz * uz)));
        f0x = f32_trunc(r0x); f0y = f32_trunc(r0y); f0z = f32_trunc(r0z);
        n0 = norm32_lo(f0x, f0y, f0z);
        set_best_up();
    }
    // step i (1-based) of length dt (negative), h = dt / 2
    __device__ __forceinline__ void step(int i, double dt, double h) {
        a.kdk(dt, h);
        b.kdk(dt, h);
        const double r1x = a.x - b.x, r1y = a.y - b.y, r1z = a.z - b.z;
        const float f1x = f32_trunc(r1x), f1y = f32_trunc(r1y), f1z = f32_trunc(r1z);
        const float n1 = norm32_lo(f1x, f1y, f1z);
        const float dn = fmaf(2.2e-7f, n0 + n1, norm32_hi(f1x - f0x, f1y - f0y, f1z - f0z));
        const float lb = (fminf(n0, n1) - 0.5f * dn) * (1.f - 1e-6f) - 1e-12f * (n0 + n1);
        if (!(lb > best_up)) {
            // the reference's segment test (seg_min and its strict comparison), with its own cheap pre-test
            const double dx = r1x - r0x, dy = r1y - r0y, dz = r1z - r0z;
            const double dd = fma(dx, dx, fma(dy, dy, dz * dz));
            const double an = fma(r0x, dx, fma(r0y, dy, r0z * dz));
            const double r0s = fma(r0x, r0x, fma(r0y, r0y, r0z * r0z));
            const double r1s = fma(r1x, r1x, fma(r1y, r1y, r1z * r1z));
            const double best2 = best * best;
            double near2dd;
            if (!(dd > 0) || an >= 0) near2dd = r0s * dd;
            else if (-an >= dd) near2dd = r1s * dd;
            else near2dd = fma(r0s, dd, -an * an);
            if (near2dd < best2 * dd * (1.0 + 1e-12) || (!(dd > 0) && r0s < best2 * (1.0 + 1e-12))) {
                double s = 0.0;
                if (dd > 0) {
                    s = -an / dd;
                    s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
                }
                const double mx = fma(dx, s, r0x), my = fma(dy, s, r0y), mz = fma(dz, s, r0z);
                const double dm = sqrt(fma(mx, mx, fma(my, my, mz * mz)));
                if (dm < best) {
                    best = dm;
                    tbest = ((double)(i - 1) + s) * -dt;
                    const double wx = a.vx - b.vx, wy = a.vy - b.vy, wz = a.vz - b.vz;
                    vbest = sqrt(fma(wx, wx, fma(wy, wy, wz * wz)));
                    set_best_up();
                }
            }
        }
        r0x = r1x; r0y = r1y; r0z = r1z;
        f0x = f1x; f0y = f1y; f0z = f1z;
        n0 = n1;
    }
};

__device__ __forceinline__ void trace_clone(const double *__restrict__ ps, int steps, double dt, double &best_o,
                                            double &tbest_o, double &vbest_o) {
    Clone c;
    c.start(ps);
    const double h = 0.5 * dt;
#pragma unroll 1
    for (int i = 1; i <= steps; i++) c.step(i, dt, h);
    best_o = c.best;
    tbest_o = c.tbest;
    vbest_o = c.vbest;
}

// ---- reduction of one pair (m clones) ---------------------------------------------------------------------------
// All sorted quantities are non-negative doubles, whose IEEE bit patterns order like their values, so the sort
// runs on 64-bit integer keys (the integer pipe; a double compare would occupy the scarce FP64 pipe).
__device__ __forceinline__ unsigned long long kmin(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
__device__ __forceinline__ unsigned long long kmax(unsigned long long a, unsigned long long b) { return a < b ? b : a; }

// bitonic sort of 32*R keys held by one warp, element e = 32*r + lane in register r: stages whose partner distance
// j is below 32 exchange across lanes with shuffles, the others swap registers within a lane
template <int R>
__device__ __forceinline__ void warp_bitonic(unsigned long long (&a)[R], int lane) {
#pragma unroll
    for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int jr = j >> 5;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    if (r & jr) continue;
                    const bool asc = ((32 * r) & k) == 0;
                    const unsigned long long lo = kmin(a[r], a[r | jr]), hi = kmax(a[r], a[r | jr]);
                    a[r] = asc ? lo : hi;
                    a[r | jr] = asc ? hi : lo;
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const unsigned long long p = __shfl_xor_sync(0xffffffffu, a[r], j);
                    const bool asc = ((32 * r + lane) & k) == 0, lower = (lane & j) == 0;
                    a[r] = (asc == lower) ? kmin(a[r], p) : kmax(a[r], p);
                }
            }
        }
    }
}

// linear-interpolated quantile of a sorted array (reference quantile, src/phygas.c:175-180), without contraction
__device__ __forceinline__ double interp_q(const double *v, int n, double q) {
    const double pos = __dmul_rn(q, (double)(n - 1));
    const int i = (int)pos;
    if (i >= n - 1) return v[n - 1];
    return __dadd_rn(v[i], __dmul_rn(__dsub_rn(pos, (double)i), __dsub_rn(v[i + 1], v[i])));
}

// one warp reduces one pair: cres holds best/tbest/vbest of its m clones (m <= 32*R)
template <int R>
__device__ void warp_reduce_pair(const double *__restrict__ best, const double *__restrict__ tbest,
                                 const double *__restrict__ vbest, int m, double r50_pc, double rtot_pc,
                                 double *smem_w, PhResultDev *out, int lane) {
    unsigned long long a[R];
    int in50 = 0, intot = 0;
    double res[9];
#pragma unroll 1
    for (int which = 0; which < 3; which++) {
        const double *src = which == 0 ? best : (which == 1 ? tbest : vbest);
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int e = 32 * r + lane;
            double v = 0.0;
            if (e < m) {
                v = __ldcg(src + e);
                if (which == 0) {
                    v = __dmul_rn(v, 1000.0);
                    in50 += v < r50_pc;
                    intot += v < rtot_pc;
                } else if (which == 2) {
                    v = __dmul_rn(v, kKms);
                }
            }
            a[r] = e < m ? (unsigned long long)__double_as_longlong(v) : 0x7ff0000000000000ULL;
        }
        warp_bitonic<R>(a, lane);
#pragma unroll
        for (int r = 0; r < R; r++) smem_w[32 * r + lane] = __longlong_as_double((long long)a[r]);
        __syncwarp();
        if (lane == 0) {
            res[3 * which + 0] = interp_q(smem_w, m, 0.05);
            res[3 * which + 1] = interp_q(smem_w, m, 0.5);
            res[3 * which + 2] = interp_q(smem_w, m, 0.95);
        }
        __syncwarp();
    }
    in50 = __reduce_add_sync(0xffffffffu, in50);
    intot = __reduce_add_sync(0xffffffffu, intot);
    if (lane == 0) {
        PhResultDev o;
        o.n = m;
        o.pad = 0;
        o.d05 = res[0]; o.d50 = res[1]; o.d95 = res[2];
        o.t05 = res[3]; o.t50 = res[4]; o.t95 = res[5];
        o.v05 = res[6]; o.v50 = res[7]; o.v95 = res[8];
        o.f_r50 = m > 0 ? __ddiv_rn((double)in50, (double)m) : 0.0;
        o.f_rtot = m > 0 ? __ddiv_rn((double)intot, (double)m) : 0.0;
        if (m <= 0) { o.d05 = o.d50 = o.d95 = o.t05 = o.t50 = o.t95 = o.v05 = o.v50 = o.v95 = 0.0; }
        *out = o;
    }
}

__device__ void reduce_dispatch(const McPairs &P, int p, double *smem_w, int lane) {
    const int m = P.clone_off[p + 1] - P.clone_off[p];
    const size_t o = P.clone_off[p];
    const double *b = P.cres + o, *t = P.cres + P.n_clones + o, *v = P.cres + 2 * (size_t)P.n_clones + o;
    PhResultDev *out = P.res + p;
    const double r50 = P.r50_pc[p], rt = P.rtot_pc[p];
    if (m <= 32) warp_reduce_pair<1>(b, t, v, m, r50, rt, smem_w, out, lane);
    else if (m <= 64) warp_reduce_pair<2>(b, t, v, m, r50, rt, smem_w, out, lane);
    else if (m <= 128) warp_reduce_pair<4>(b, t, v, m, r50, rt, smem_w, out, lane);
    else if (m <= 256) warp_reduce_pair<8>(b, t, v, m, r50, rt, smem_w, out, lane);
    else if (m <= 512) warp_reduce_pair<16>(b, t, v, m, r50, rt, smem_w, out, lane);
    else warp_reduce_pair<32>(b, t, v, m, r50, rt, smem_w, out, lane);
}

// Persistent clone kernel.  items[q] = (pair, first clone, count <= 32), longest trace first.  No warp ever waits
// for another: a warp takes the next item with one atomic, and the warp whose item completes a pair's count (an
// atomic per item, after a fence) reduces that pair.
__global__ void __launch_bounds__(kMcThreads) k_pair_mc(McPairs P) {
    __shared__ double smem[kMcThreads / 32][1024];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(P.qhead, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= P.n_items) break;
        const int4 it = P.items[q];   // x = pair, y = first clone, z = count
        const int p = it.x;
        if (lane < it.z) {
            const int c = it.y + lane;
            double best, tbest, vbest;
            trace_clone(P.ps + (size_t)c * 12, P.steps[p], P.dt[p], best, tbest, vbest);
            P.cres[c] = best;
            P.cres[P.n_clones + c] = tbest;
            P.cres[2 * (size_t)P.n_clones + c] = vbest;
        }
        __threadfence();
        __syncwarp();
        int last = 0;
        if (lane == 0) {
            const int m = P.clone_off[p + 1] - P.clone_off[p];
            last = atomicAdd(P.done + p, it.z) + it.z == m;
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (last) {
            __threadfence();
            const int m = P.clone_off[p + 1] - P.clone_off[p];
            if (m <= 1024) reduce_dispatch(P, p, smem[w], lane);
        }
    }
}

// Persistent clone tracing for batches replayed from a captured graph: parameters read from device memory, and the
// launch shape a template: WARPS warps per block, CPL clones per lane traced in lockstep (items of up to 32 * CPL
// clones; a lane past its item's end repeats its first clone and discards the copy), and MINB resident blocks per SM
// asked of the compiler (fewer registers per thread, more warps to hide the FP64 pipe's latency).  Tracing only -- the pairs are
// reduced by k_pair_reduce_dev afterwards, which keeps this kernel's registers to the orbits'.  The clones'
// arithmetic is the same in every variant, so every variant gives the same bits.
template <int WARPS, int CPL, int MINB>
__global__ void __launch_bounds__(WARPS * 32, MINB) k_pair_mc_t(const McPairs *__restrict__ Pd) {
    const McPairs P = *Pd;
    const int lane = threadIdx.x & 31;
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(P.qhead, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= P.n_items) break;
        const int4 it = P.items[q];   // x = pair, y = first clone, z = count
        if (lane >= it.z) continue;
        const int p = it.x;
        const int steps = P.steps[p];
        const double dt = P.dt[p], h = 0.5 * dt;
        Clone c[CPL];
#pragma unroll
        for (int j = 0; j < CPL; j++) {
            const int e = lane + 32 * j < it.z ? lane + 32 * j : lane;
            c[j].start(P.ps + (size_t)(it.y + e) * 12);
        }
#pragma unroll 1
        for (int i = 1; i <= steps; i++) {
#pragma unroll
            for (int j = 0; j < CPL; j++) c[j].step(i, dt, h);
        }
#pragma unroll
        for (int j = 0; j < CPL; j++) {
            if (lane + 32 * j >= it.z) continue;
            const int cc = it.y + lane + 32 * j;
            P.cres[cc] = c[j].best;
            P.cres[P.n_clones + cc] = c[j].tbest;
            P.cres[2 * (size_t)P.n_clones + cc] = c[j].vbest;
        }
    }
}

// before k_pair_mc_t: queue head zeroed, empty results for pairs without clones
__global__ void k_mc_prep(const McPairs *__restrict__ Pd) {
    const McPairs P = *Pd;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) *P.qhead = 0;
    for (int p = t; p < P.n_pairs; p += gridDim.x * blockDim.x) {
        if (P.clone_off[p + 1] - P.clone_off[p] > 0) continue;
        PhResultDev o;
        o.n = 0;
        o.pad = 0;
        o.d05 = o.d50 = o.d95 = o.t05 = o.t50 = o.t95 = o.v05 = o.v50 = o.v95 = o.f_r50 = o.f_rtot = 0.0;
        P.res[p] = o;
    }
}

// after k_pair_mc_t: one warp per pair of 1 .. 1024 clones, over a fixed grid
__global__ void __launch_bounds__(kMcThreads) k_pair_reduce_dev(const McPairs *__restrict__ Pd) {
    __shared__ double smem[kMcThreads / 32][1024];
    const McPairs P = *Pd;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int p = blockIdx.x * (kMcThreads / 32) + w; p < P.n_pairs; p += gridDim.x * (kMcThreads / 32)) {
        const int m = P.clone_off[p + 1] - P.clone_off[p];
        if (m > 0 && m <= 1024) reduce_dispatch(P, p, smem[w], lane);
    }
}

namespace {
struct McVariant {
    int warps, cpl, min_blocks;
    void (*fn)(const McPairs *);
};
const McVariant kMcVariants[] = {
    {4, 1, 1, k_pair_mc_t<4, 1, 1>}, {2, 1, 1, k_pair_mc_t<2, 1, 1>}, {8, 1, 1, k_pair_mc_t<8, 1, 1>},
    {4, 2, 1, k_pair_mc_t<4, 2, 1>}, {2, 2, 1, k_pair_mc_t<2, 2, 1>}, {8, 2, 1, k_pair_mc_t<8, 2, 1>},
    {4, 1, 5, k_pair_mc_t<4, 1, 5>}, {4, 1, 6, k_pair_mc_t<4, 1, 6>}, {8, 1, 3, k_pair_mc_t<8, 1, 3>},
};
}  // namespace

int mc_variants() { return (int)(sizeof kMcVariants / sizeof kMcVariants[0]); }

void mc_variant_shape(int v, int &warps, int &cpl, int &min_blocks) {
    warps = kMcVariants[v].warps;
    cpl = kMcVariants[v].cpl;
    min_blocks = kMcVariants[v].min_blocks;
}

// resident blocks of variant v for a full persistent grid (blocks per SM x SMs)
cudaError_t mc_variant_grid(int v, int sms, int &grid) {
    int per_sm = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, reinterpret_cast<const void *>(kMcVariants[v].fn), kMcVariants[v].warps * 32, 0);
    grid = sms * (per_sm > 0 ? per_sm : 1);
    return e;
}

// prep, trace (variant v on a persistent grid) and reduce on one stream; reduce_grid blocks of kMcThreads
cudaError_t launch_mc(int v, int grid, int prep_grid, int reduce_grid, cudaStream_t st, const McPairs *Pd) {
    k_mc_prep<<<prep_grid, 256, 0, st>>>(Pd);
    kMcVariants[v].fn<<<grid, kMcVariants[v].warps * 32, 0, st>>>(Pd);
    k_pair_reduce_dev<<<reduce_grid, kMcThreads, 0, st>>>(Pd);
    return cudaGetLastError();
}

// reduction alone, one warp per pair, for results traced elsewhere (the drop-in ph_pair_reduce)
__global__ void __launch_bounds__(kMcThreads) k_pair_reduce_only(McPairs P) {
    __shared__ double smem[kMcThreads / 32][1024];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int p = blockIdx.x * (kMcThreads / 32) + w;
    if (p >= P.n_pairs) return;
    const int m = P.clone_off[p + 1] - P.clone_off[p];
    if (m > 0 && m <= 1024) reduce_dispatch(P, p, smem[w], lane);
}

// A pair's clone value e of array `which` (0 best, 1 tbest, 2 vbest) in the units of the reduction, as the bit
// pattern that orders it: the values are non-negative, so their IEEE patterns sort as unsigned integers.
__device__ __forceinline__ unsigned long long reduce_key(const double *src, int which, int e) {
    double v = src[e];
    if (which == 0) v = __dmul_rn(v, 1000.0);
    else if (which == 2) v = __dmul_rn(v, kKms);
    return (unsigned long long)__double_as_longlong(v);
}

// The k-th smallest (0-based) of a pair's m values of array `which`, read from global memory by the whole block: an
// MSB radix selection, 8 bits a pass, each pass counting the values that share the prefix found so far.  Exact: the
// element a sort would put at index k.  For pairs too large to sort in shared memory.
__device__ double radix_select(const double *src, int which, int m, int k) {
    __shared__ unsigned hist[256];
    __shared__ unsigned long long s_prefix;
    __shared__ int s_k;
    if (threadIdx.x == 0) { s_prefix = 0; s_k = k; }
    unsigned long long mask = 0;
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
        __syncthreads();
        const unsigned long long prefix = s_prefix;
        for (int e = threadIdx.x; e < m; e += blockDim.x) {
            const unsigned long long key = reduce_key(src, which, e);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int kk = s_k, b = 0;
            for (; b < 255 && kk >= (int)hist[b]; b++) kk -= (int)hist[b];
            s_k = kk;
            s_prefix = prefix | ((unsigned long long)b << shift);
        }
        mask |= 255ull << shift;
        __syncthreads();
    }
    const double v = __longlong_as_double((long long)s_prefix);
    __syncthreads();
    return v;
}

// interp_q of the sorted values, the two order statistics it reads found by radix_select
__device__ double select_q(const double *src, int which, int m, double q) {
    const double pos = __dmul_rn(q, (double)(m - 1));
    const int i = (int)pos;
    if (i >= m - 1) return radix_select(src, which, m, m - 1);
    const double a = radix_select(src, which, m, i), b = radix_select(src, which, m, i + 1);
    return __dadd_rn(a, __dmul_rn(__dsub_rn(pos, (double)i), __dsub_rn(b, a)));
}

// pairs of 0 clones never get an item: their (empty) result is written here, with the big-pair reduction.  Pairs of
// up to kSortMax clones are sorted in shared memory (launched with room for the batch's largest such pair); larger
// pairs take their order statistics by radix selection from global memory.
__global__ void k_pair_reduce_big(McPairs P) {
    extern __shared__ double sm[];
    const int p = blockIdx.x;
    const int m = P.clone_off[p + 1] - P.clone_off[p];
    if (m > 0 && m <= 1024) return;
    PhResultDev *out = P.res + p;
    if (m <= 0) {
        if (threadIdx.x == 0) {
            PhResultDev o;
            o.n = 0;
            o.pad = 0;
            o.d05 = o.d50 = o.d95 = o.t05 = o.t50 = o.t95 = o.v05 = o.v50 = o.v95 = o.f_r50 = o.f_rtot = 0.0;
            *out = o;
        }
        return;
    }
    int n2 = 1;
    while (n2 < m) n2 <<= 1;
    unsigned long long *key = reinterpret_cast<unsigned long long *>(sm);
    const size_t o = P.clone_off[p];
    __shared__ int c50, ctot;
    __shared__ double res[9];
    if (threadIdx.x == 0) { c50 = 0; ctot = 0; }
    __syncthreads();
    if (m > kSortMax) {
        int l50 = 0, ltot = 0;
        for (int e = threadIdx.x; e < m; e += blockDim.x) {
            const double v = __dmul_rn(P.cres[o + e], 1000.0);
            l50 += v < P.r50_pc[p];
            ltot += v < P.rtot_pc[p];
        }
        atomicAdd(&c50, l50);
        atomicAdd(&ctot, ltot);
        for (int which = 0; which < 3; which++) {
            const double *src = P.cres + (size_t)which * P.n_clones + o;
            const double q05 = select_q(src, which, m, 0.05), q50 = select_q(src, which, m, 0.5),
                         q95 = select_q(src, which, m, 0.95);
            if (threadIdx.x == 0) { res[3 * which] = q05; res[3 * which + 1] = q50; res[3 * which + 2] = q95; }
        }
        __syncthreads();
        n2 = 0;                             // nothing left to sort below
    }
    for (int which = 0; which < 3 && n2 > 0; which++) {
        const double *src = P.cres + (size_t)which * P.n_clones + o;
        int l50 = 0, ltot = 0;
        for (int e = threadIdx.x; e < n2; e += blockDim.x) {
            double v = 0.0;
            if (e < m) {
                v = src[e];
                if (which == 0) { v = __dmul_rn(v, 1000.0); l50 += v < P.r50_pc[p]; ltot += v < P.rtot_pc[p]; }
                else if (which == 2) v = __dmul_rn(v, kKms);
            }
            key[e] = e < m ? (unsigned long long)__double_as_longlong(v) : 0x7ff0000000000000ULL;
        }
        if (which == 0) { atomicAdd(&c50, l50); atomicAdd(&ctot, ltot); }
        __syncthreads();
        for (int k = 2; k <= n2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int e = threadIdx.x; e < n2; e += blockDim.x) {
                    const int f = e ^ j;
                    if (f > e) {
                        const unsigned long long x = key[e], y = key[f];
                        const bool asc = (e & k) == 0;
                        if ((x > y) == asc) { key[e] = y; key[f] = x; }
                    }
                }
                __syncthreads();
            }
        if (threadIdx.x == 0) {
            const double *v = reinterpret_cast<const double *>(key);
            res[3 * which] = interp_q(v, m, 0.05);
            res[3 * which + 1] = interp_q(v, m, 0.5);
            res[3 * which + 2] = interp_q(v, m, 0.95);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        PhResultDev r;
        r.n = m;
        r.pad = 0;
        r.d05 = res[0]; r.d50 = res[1]; r.d95 = res[2];
        r.t05 = res[3]; r.t50 = res[4]; r.t95 = res[5];
        r.v05 = res[6]; r.v50 = res[7]; r.v95 = res[8];
        r.f_r50 = __ddiv_rn((double)c50, (double)m);
        r.f_rtot = __ddiv_rn((double)ctot, (double)m);
        *out = r;
    }
}

}  // namespace pgx

namespace pgx {
// Peak-rate probes for the roofline denominators (FP64 and FP32 are not in the driver's measured peaks): long
// independent FMA chains, 8 per thread; the result is stored so nothing is eliminated.
__global__ void k_peak_dfma(double *out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
    double s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_peak_ffma(float *out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fmaf(x[i], a, b);
    float s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace pgx

// ---------------------------------------------------------------------------------------------------------------
// pgx_pair_noalloc: the pair Monte Carlo for callers that cannot allocate GPU memory.
//
// Some callers may not call cudaMalloc at all: code that runs inside another framework's memory pool (the pool
// owns the device memory and a stray allocation fragments it or fails), real-time loops that must not stall on the
// allocator, and host code that hands this library only the device buffers it already has.  This entry point takes
// the caller's device buffers for inputs and outputs and keeps its own scratch -- the per-clone closest approaches
// and the work-queue head -- in a fixed array compiled into the library (static __device__ storage, held by every
// GPU that loads the library until the process exits).  It calls no allocating routine.
//
// Limits: at most kNoAllocMaxClones clones per call (24 MiB of scratch); pairs of more than 1024 clones get a result
// with n = -1 (pgx_pair handles them), and so does a pair whose offsets leave [0, n_clones).  Every call shares the
// one scratch array and leaves its contents behind; two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.  The first call on a device runs the
// set-up below, which fills the force tables with a kernel on the legacy default stream and synchronizes the whole
// device: make it before any stream capture, and outside latency-critical work.
namespace pgx {

constexpr int kNoAllocMaxClones = 1 << 20;

// per-clone results: best (kpc), tbest (Myr), vbest (kpc/Myr), each kNoAllocMaxClones long
static __device__ __align__(256) double g_noalloc_cres[3 * kNoAllocMaxClones];
// work-queue head (cleared at the start of every call)
static __device__ __align__(256) int g_noalloc_qhead[64];

// persistent: warps take chunks of 32 consecutive clones; a lane finds its clone's pair by binary search
__global__ void __launch_bounds__(kMcThreads) k_pair_mc_noalloc(int n_pairs, int n_clones,
                                                                const int *__restrict__ clone_off,
                                                                const double *__restrict__ ps,
                                                                const int *__restrict__ steps,
                                                                const double *__restrict__ dt, double *cres, int *qhead) {
    const int lane = threadIdx.x & 31;
    const int n_chunks = (n_clones + 31) / 32;
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(qhead, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= n_chunks) break;
        const int c = q * 32 + lane;
        if (c < n_clones) {
            int lo = 0, hi = n_pairs;          // clone_off[lo] <= c < clone_off[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (clone_off[mid] <= c) lo = mid; else hi = mid;
            }
            double b, t, v;
            trace_clone(ps + (size_t)c * 12, steps[lo], dt[lo], b, t, v);
            cres[c] = b;
            cres[kNoAllocMaxClones + c] = t;
            cres[2 * (size_t)kNoAllocMaxClones + c] = v;
        }
    }
}

// one warp per pair, after all clones are traced (stream order).  The offsets are device memory the host cannot
// check: a pair whose clones do not lie inside [0, n_clones) -- the clones this call traced -- gets n = -1 instead
// of reading scratch the call did not write (or memory past it).
__global__ void __launch_bounds__(kMcThreads) k_pair_reduce_noalloc(int n_pairs, int n_clones,
                                                                    const int *__restrict__ clone_off,
                                                                    const double *__restrict__ r50,
                                                                    const double *__restrict__ rt,
                                                                    const double *cres, PhResultDev *res) {
    __shared__ double smem[kMcThreads / 32][1024];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int p = blockIdx.x * (kMcThreads / 32) + w;
    if (p >= n_pairs) return;
    const int o = clone_off[p], e = clone_off[p + 1];
    const bool bad = o < 0 || e < o || e > n_clones;
    const int m = bad ? -1 : e - o;
    if (m <= 0 || m > 1024) {
        if (lane == 0) {
            PhResultDev z;
            z.n = m == 0 ? 0 : -1;
            z.pad = 0;
            z.d05 = z.d50 = z.d95 = z.t05 = z.t50 = z.t95 = z.v05 = z.v50 = z.v95 = z.f_r50 = z.f_rtot = 0.0;
            res[p] = z;
        }
        return;
    }
    const double *b = cres + o, *t = cres + kNoAllocMaxClones + o, *v = cres + 2 * (size_t)kNoAllocMaxClones + o;
    if (m <= 32) warp_reduce_pair<1>(b, t, v, m, r50[p], rt[p], smem[w], res + p, lane);
    else if (m <= 64) warp_reduce_pair<2>(b, t, v, m, r50[p], rt[p], smem[w], res + p, lane);
    else if (m <= 128) warp_reduce_pair<4>(b, t, v, m, r50[p], rt[p], smem[w], res + p, lane);
    else if (m <= 256) warp_reduce_pair<8>(b, t, v, m, r50[p], rt[p], smem[w], res + p, lane);
    else if (m <= 512) warp_reduce_pair<16>(b, t, v, m, r50[p], rt[p], smem[w], res + p, lane);
    else warp_reduce_pair<32>(b, t, v, m, r50[p], rt[p], smem[w], res + p, lane);
}

namespace {
// set-up, once per device: the device addresses of the scratch arrays (in host code their names are host-side
// stand-ins, not device addresses) and the persistent grid size
struct NoAllocDevice {
    double *cres = nullptr;
    int *qhead = nullptr;
    int grid = 0;
    bool ready = false;
};
NoAllocDevice g_noalloc_dev[64];
std::mutex g_noalloc_mu;

int noalloc_setup(int dev, NoAllocDevice *&out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        cudaError_t e = orbit_setup(dev) ? cudaErrorUnknown : cudaSuccess;
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&d.cres, g_noalloc_cres);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&d.qhead, g_noalloc_qhead);
        int sms = 0, per_sm = 0;
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pair_mc_noalloc, kMcThreads, 0);
        if (e != cudaSuccess) {
            fprintf(stderr, "pgx_pair_noalloc: set-up on device %d failed: %s\n", dev, cudaGetErrorString(e));
            return PGX_E_CUDA;
        }
        d.grid = sms * (per_sm > 0 ? per_sm : 1);
        d.ready = true;
    }
    out = &d;
    return 0;
}
}  // namespace
}  // namespace pgx

extern "C" int pgx_pair_noalloc(void *stream, int n_pairs, int n_clones, const int *clone_off, const double *ps,
                                const int *steps, const double *dt, const double *r50_pc, const double *rtot_pc,
                                PhResult *res) {
    if (n_pairs < 0 || n_clones < 0 || (n_pairs > 0 && (!clone_off || !steps || !dt || !r50_pc || !rtot_pc || !res)) ||
        (n_clones > 0 && !ps)) {
        fprintf(stderr, "pgx_pair_noalloc: invalid arguments\n");
        return PGX_E_ARG;
    }
    if (n_clones > pgx::kNoAllocMaxClones) {
        fprintf(stderr, "pgx_pair_noalloc: %d clones in one call; its fixed scratch holds %d (use pgx_pair)\n",
                n_clones, pgx::kNoAllocMaxClones);
        return PGX_E_LIMIT;
    }
    if (n_pairs == 0) return 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        fprintf(stderr, "pgx_pair_noalloc: no current device (%s)\n", cudaGetErrorString(e));
        return PGX_E_NODEV;
    }
    pgx::NoAllocDevice *d = nullptr;
    int rc = pgx::noalloc_setup(dev, d);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    e = cudaMemsetAsync(d->qhead, 0, sizeof(int), st);
    if (e == cudaSuccess && n_clones > 0) {
        const int grid = std::max(1, std::min(d->grid, (n_clones + 127) / 128));
        pgx::k_pair_mc_noalloc<<<grid, pgx::kMcThreads, 0, st>>>(n_pairs, n_clones, clone_off, ps, steps, dt,
                                                                  d->cres, d->qhead);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        const int wpb = pgx::kMcThreads / 32;
        pgx::k_pair_reduce_noalloc<<<(n_pairs + wpb - 1) / wpb, pgx::kMcThreads, 0, st>>>(
            n_pairs, n_clones, clone_off, r50_pc, rtot_pc, d->cres, reinterpret_cast<pgx::PhResultDev *>(res));
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        fprintf(stderr, "pgx_pair_noalloc: launch failed: %s\n", cudaGetErrorString(e));
        return PGX_E_CUDA;
    }
    return 0;
}

namespace pgx {
// The halo power tables of pgx_force.cuh, filled once per device (before the first orbit kernel on it; call it
// outside any stream capture).
int orbit_setup(int dev) {
    static std::mutex mu;
    static bool ready[64] = {};
    if (dev < 0 || dev >= 64) return 1;
    std::lock_guard<std::mutex> lk(mu);
    if (ready[dev]) return 0;
    long long b1, b2;                       // the force compares these bit patterns as integers
    std::memcpy(&b1, &kHaloCut, 8);
    std::memcpy(&b2, &kTinyR2, 8);
    if (b1 != kHaloCutBits || b2 != kTinyR2Bits) return 3;
    k_halo_tables<<<1, kHaloTableThreads>>>();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return 2;
    ready[dev] = true;
    return 0;
}
}  // namespace pgx
