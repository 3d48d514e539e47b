// pgx_text.h -- screen rows as text on the GPU (internal header).
#pragma once
#include <string>
#include "pgx_mixed.h"

namespace pgx {

constexpr long kTextBatch = 4 << 20;        // rows per batch: 4Mi lines of at most kFmtMaxRow bytes fit an int offset
constexpr int kFmtMaxRow = 2 * 40 + 4 + 9 * 331;   // two names, kind, spaces, nine numbers, newline (upper bound)

struct TextLabels {
    const char *ids;                 // 40 bytes per star of the chunk
    const char *names;               // 40 bytes per cluster
    const char *kinds;               // one per cluster
    const double *age16, *age84;     // per cluster
};

struct TextBufs {
    DevBuf len, off, part;
};

// rows[0, n) as text into out (device, cap bytes): *bytes = the text's length; PGX_E_LIMIT with *bytes = a size that
// suffices when cap is too small
int format_rows(cudaStream_t st, long n, const ScreenRowDev *rows, const TextLabels &L, TextBufs &b, char *out,
                size_t cap, size_t *bytes, std::string &err);
void text_free(TextBufs &b);

}  // namespace pgx
