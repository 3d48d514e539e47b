// pgx_mixed.cu -- mixed-precision screen of libphygas_gb300 and the cluster-table column gather.
#include <vector>
#include "pgx_internal.cuh"
#include "pgx_mixed.h"
#include "pgx_screen_math.cuh"

namespace pgx {

namespace {
int grow(DevBuf &b, size_t bytes, std::string &err) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return 0;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes + bytes / 4);
    if (e != cudaSuccess) {
        err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PGX_E_NOMEM : PGX_E_CUDA;
    }
    b.cap = bytes + bytes / 4;
    return 0;
}
int check(cudaError_t e, std::string &err, const char *what) {
    if (e == cudaSuccess) return 0;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return PGX_E_CUDA;
}
}  // namespace

void mixed_free(MixedBufs &m) {
    DevBuf *all[] = {&m.order, &m.ub, &m.flag, &m.cnt, &m.off, &m.total, &m.kept, &m.cand, &m.cand_off,
                     &m.ent, &m.entq, &m.aux};
    for (DevBuf *b : all)
        if (b->p) { cudaFree(b->p); b->p = nullptr; b->cap = 0; }
}

__global__ void k_gather_cols(int nc, int nmax, const int *__restrict__ order, const double *__restrict__ s64,
                              const float4 *__restrict__ s32, double *__restrict__ d64, float4 *__restrict__ d32) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)nc * nmax) return;
    const int slot = (int)(idx % nc), k = (int)(idx / nc), col = order[slot];
    const size_t NC = nc;
    for (int f = 0; f < 12; f++) d64[((size_t)k * 12 + f) * NC + col] = s64[((size_t)k * 12 + f) * NC + slot];
    for (int q = 0; q < 3; q++) d32[((size_t)k * NC + col) * 3 + q] = s32[((size_t)k * NC + slot) * 3 + q];
}

int gather_columns(cudaStream_t st, int nc, int nmax, const int *order_host, const double *t64_slot,
                   const float4 *t32_slot, double *c64, float4 *c32, MixedBufs &m) {
    int rc = grow(m.order, (size_t)nc * 4, m.err);
    if (rc) return rc;
    if ((rc = check(cudaMemcpyAsync(m.order.p, order_host, (size_t)nc * 4, cudaMemcpyHostToDevice, st), m.err, "order")))
        return rc;
    if ((rc = check(cudaMemsetAsync(c64, 0, (size_t)nmax * 12 * nc * 8, st), m.err, "memset"))) return rc;
    if ((rc = check(cudaMemsetAsync(c32, 0, (size_t)nmax * 3 * nc * 16, st), m.err, "memset"))) return rc;
    const size_t work = (size_t)nc * nmax;
    k_gather_cols<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(nc, nmax, (const int *)m.order.p, t64_slot, t32_slot,
                                                                   c64, c32);
    if ((rc = check(cudaGetLastError(), m.err, "k_gather_cols"))) return rc;
    // the host order array must outlive the async copy
    return check(cudaStreamSynchronize(st), m.err, "gather sync");
}

int mixed_cluster_aux(cudaStream_t, int, int, const float4 *, const int *, const double *, MixedBufs &) { return 0; }

int mixed_select(cudaStream_t, const ScreenTables &, double, MixedBufs &m, cudaEvent_t, int *, PgxStats *) {
    m.err = "mixed-precision screen not built in this version";
    return PGX_E_ARG;
}
const KeptPair *mixed_kept(MixedBufs &m) { return (const KeptPair *)m.kept.p; }
int mixed_finish(cudaStream_t, int, const FinishIn *, ScreenRowDev *, MixedBufs &m, PgxStats *) {
    m.err = "mixed-precision finish not built in this version";
    return PGX_E_ARG;
}

}  // namespace pgx
