// Host planning of the dense sweep in C++ (no GPU): the op stream of one query from the span-form
// constraint rows and the reduced target row (the loop of cdist/trellis.py:147-182, in the order of
// tropidist_gb300/trellis.py make_plan).  Rows are bitsets over column positions.
#include "tg_common.cuh"
#include "tg_capi.h"

#include <algorithm>
#include <vector>

using namespace tg;

extern "C" {

// rows: nrows bitsets of `words` uint64 each (position j = bit j % 64 of word j / 64), the target
// row last (it is row nrows - 1 and selects to 1, all others to 0); weights: per-position column
// weight or NULL (unit).  ops: int64 [cap][3] rows (0,0,0) expand / (1, mask, w) update / (2, pos,
// target) select; widths: int32 [ncols] active rows after each position; columns: int32 [cap] the
// position of each update.  out: [0] ops, [1] updates, [2] peak width.  Returns 0, -1 on bad
// arguments, -4 when a mask needs more than 63 rows, or the op count needed (> cap) when ops do not
// fit (nothing is then written past cap).
int tg_make_plan(int nrows, int ncols, int words, const uint64_t *rows, const int64_t *weights, int64_t *ops,
                 int64_t cap, int32_t *widths, int32_t *columns, int64_t *out) {
    if (nrows < 1 || ncols < 0 || words < (ncols + 63) / 64 || !rows || !ops || !widths || !columns || !out)
        return set_error(TG_ERR_ARG, "bad plan rows");
    auto bit = [&](int r, int j) { return (rows[(size_t)r * words + (j >> 6)] >> (j & 63)) & 1ull; };
    // first and last position of every row
    std::vector<std::vector<int>> begins((size_t)ncols + 1), finishes((size_t)ncols + 1);
    for (int r = 0; r < nrows; r++) {
        int lo = -1, hi = -1;
        for (int w = 0; w < words; w++) {
            const uint64_t x = rows[(size_t)r * words + w];
            if (!x) continue;
            if (lo < 0) lo = w * 64 + __builtin_ctzll(x);
            hi = w * 64 + 63 - __builtin_clzll(x);
        }
        if (lo < 0) continue;                         // an empty row never becomes active
        if (hi >= ncols) return set_error(TG_ERR_ARG, "row beyond the columns");
        begins[(size_t)lo].push_back(r);
        finishes[(size_t)hi].push_back(r);
    }
    std::vector<int> active;
    int64_t n = 0, nupd = 0;
    int peak = 0;
    auto emit = [&](int64_t a, int64_t b, int64_t c) {
        if (n < cap) { ops[3 * n] = a; ops[3 * n + 1] = b; ops[3 * n + 2] = c; }
        n++;
    };
    for (int j = 0; j < ncols; j++) {
        for (int r : begins[(size_t)j]) {
            active.push_back(r);
            emit(0, 0, 0);
        }
        if ((int)active.size() > peak) peak = (int)active.size();
        uint64_t mask = 0;
        for (size_t pos = 0; pos < active.size(); pos++)
            if (bit(active[pos], j)) {
                if (pos >= 63) return set_error(TG_ERR_TOO_BIG, "update masks are limited to 63 bits");
                mask |= 1ull << pos;
            }
        if (mask) {                                   // a column touching no active row is free
            emit(1, (int64_t)mask, weights ? weights[j] : 1);
            if (nupd < cap) columns[nupd] = j;
            nupd++;
        }
        // rows closing here, by position, highest first
        std::vector<int> pos_close;
        for (int r : finishes[(size_t)j])
            for (size_t pos = 0; pos < active.size(); pos++)
                if (active[pos] == r) { pos_close.push_back((int)pos); break; }
        std::sort(pos_close.begin(), pos_close.end());
        for (int k = (int)pos_close.size() - 1; k >= 0; k--) {
            const int pos = pos_close[(size_t)k];
            emit(2, pos, active[(size_t)pos] == nrows - 1 ? 1 : 0);
            active.erase(active.begin() + pos);
        }
        widths[j] = (int32_t)active.size();
    }
    if (!active.empty()) return set_error(TG_ERR_ARG, "rows left open");
    out[0] = n;
    out[1] = nupd;
    out[2] = peak;
    return n > cap ? (int)std::min<int64_t>(n, 0x7FFFFFFF) : TG_OK;
}

}  // extern "C"
