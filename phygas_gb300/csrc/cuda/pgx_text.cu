// pgx_text.cu -- the screen's rows as the reference CLI's text lines (src/phygas_screen.c:60-61), formatted on the GPU:
//   target cluster kind chi2 t_myr d_nom_pc sig_pc p_r50 p_rtot vrel_kms age16 age84
// as "%s %s %c %.3f %.3f %.2f %.2f %.4f %.4f %.2f %.3f %.3f\n", byte for byte the C library's text (pgx_fmt.cuh).
//   k_row_len   one thread per row: the line's length
//   (exclusive scan of the lengths: each line's offset)
//   k_row_text  one thread per row: the line formatted into shared memory, the block's lines written out together
// Rows go in batches of at most kTextBatch, so that a batch's offsets fit in an int.
#include <algorithm>
#include <initializer_list>

#include "pgx_fmt.cuh"
#include "pgx_mixed.h"
#include "pgx_text.h"

namespace pgx {

__device__ __forceinline__ int row_text(char *o, const ScreenRowDev &r, const TextLabels &L) {
    int n = 0;
    auto at = [&]() { return o ? o + n : nullptr; };
    auto ch = [&](char c) {
        if (o) o[n] = c;
        n++;
    };
    n += fmt_str(at(), L.ids + 40 * (size_t)r.star, 40);
    ch(' ');
    n += fmt_str(at(), L.names + 40 * (size_t)r.cluster, 40);
    ch(' ');
    ch(L.kinds[r.cluster]);
    const double v[9] = {r.chi2, r.t_myr, r.d_nom_pc, r.sig_pc, r.p_r50, r.p_rtot, r.vrel_kms, L.age16[r.cluster],
                         L.age84[r.cluster]};
    const int nd[9] = {3, 3, 2, 2, 4, 4, 2, 3, 3};
#pragma unroll 1
    for (int i = 0; i < 9; i++) {
        ch(' ');
        n += fmt_fixed(at(), v[i], nd[i]);
    }
    ch('\n');
    return n;
}

__global__ void k_row_len(int n, const ScreenRowDev *__restrict__ rows, TextLabels L, int *__restrict__ len) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < n) len[h] = row_text(nullptr, rows[h], L);
}

// A block's lines are contiguous in the output.  They are formatted into shared memory first (byte stores there are
// cheap), placed at the output's alignment modulo 16, and the block writes the span out with 16-byte stores (bytes
// at its two ends): whole sectors, where one thread per line storing bytes to global memory wrote partial sectors.
// A span too long for the staging area (lines of very large numbers) is written line by line.
constexpr int kTextRows = 128, kTextStage = 24576;

__global__ void __launch_bounds__(kTextRows) k_row_text(int n, const ScreenRowDev *__restrict__ rows, TextLabels L,
                                                        const int *__restrict__ off, const int *__restrict__ len,
                                                        char *__restrict__ out) {
    __shared__ __align__(16) char buf[kTextStage + 16];
    const int h0 = blockIdx.x * kTextRows, h = h0 + threadIdx.x, hl = min(h0 + kTextRows, n) - 1;
    const long b0 = off[h0], span = (long)off[hl] + len[hl] - b0;
    char *dst = out + b0;
    const int a = (int)((uintptr_t)dst & 15);
    if (span + a > kTextStage) {
        if (h < n) row_text(out + off[h], rows[h], L);
        return;
    }
    if (h < n) row_text(buf + a + (off[h] - b0), rows[h], L);
    __syncthreads();
    const int head = (int)min((long)((16 - a) & 15), span);
    if ((int)threadIdx.x < head) dst[threadIdx.x] = buf[a + threadIdx.x];
    const long nvec = (span - head) / 16;
    const uint4 *src4 = reinterpret_cast<const uint4 *>(buf + a + head);
    uint4 *dst4 = reinterpret_cast<uint4 *>(dst + head);
    for (long i = threadIdx.x; i < nvec; i += kTextRows) dst4[i] = src4[i];
    for (long i = head + nvec * 16 + threadIdx.x; i < span; i += kTextRows) dst[i] = buf[a + i];
}

int format_rows(cudaStream_t st, long n, const ScreenRowDev *rows, const TextLabels &L, TextBufs &b, char *out,
                size_t cap, size_t *bytes, std::string &err) {
    *bytes = 0;
    int rc;
    const int batch = (int)std::min<long>(n, kTextBatch);
    if (n == 0) return 0;
    if ((rc = grow(b.len, (size_t)batch * 4, err)) || (rc = grow(b.off, (size_t)batch * 4, err)) ||
        (rc = grow(b.part, ((size_t)batch / 1024 + 2) * 4 + 64, err)))
        return rc;
    int *len = static_cast<int *>(b.len.p), *off = static_cast<int *>(b.off.p), *part = static_cast<int *>(b.part.p);
    int *tot = part + batch / 1024 + 2;
    size_t base = 0;
    for (long h0 = 0; h0 < n; h0 += batch) {
        const int m = (int)std::min<long>(batch, n - h0);
        k_row_len<<<(m + 255) / 256, 256, 0, st>>>(m, rows + h0, L, len);
        if ((rc = check(cudaGetLastError(), err, "k_row_len"))) return rc;
        if ((rc = exclusive_scan(st, m, len, off, part, tot, err))) return rc;
        int total = 0;
        if ((rc = check(cudaMemcpyAsync(&total, tot, 4, cudaMemcpyDeviceToHost, st), err, "text total")) ||
            (rc = check(cudaStreamSynchronize(st), err, "text total sync")))
            return rc;
        if (base + (size_t)total > cap) {
            *bytes = base + (size_t)total + (size_t)(n - h0 - m) * kFmtMaxRow;     // room that suffices
            err = "text buffer too small";
            return PGX_E_LIMIT;
        }
        k_row_text<<<(m + kTextRows - 1) / kTextRows, kTextRows, 0, st>>>(m, rows + h0, L, off, len, out + base);
        if ((rc = check(cudaGetLastError(), err, "k_row_text"))) return rc;
        base += (size_t)total;
    }
    *bytes = base;
    return 0;
}

void text_free(TextBufs &b) {
    for (DevBuf *d : {&b.len, &b.off, &b.part})
        if (d->p) cudaFree(d->p);
    b = TextBufs();
}

}  // namespace pgx
