/* C port of the reference's sparse Rank DP table kernels: TEST INFRASTRUCTURE ONLY (the timed CPU
 * baseline of the sparse sweep, single-threaded as the reference's are).
 *
 *   spp_candidates   cdist/sparse_dp.c:118-157   candidates key ^ upd (value + w) of the states
 *                                                below the cap, filtered by the closing rows and the
 *                                                lookahead bound, in key order (the reference's
 *                                                default ordering: the sorted sources reordered by
 *                                                the XOR, cdist/sparse_dp.c:89-114)
 *   spp_merge        cdist/sparse_dp.c:162-202   merge by key with the filtered old table, keeping
 *                                                the smaller value; the list of changed states
 *   spp_join         cdist/sparse_dp.c:207-236   least f.value + b.value over b.key = f.key ^ tmask
 *   spp_hist         cdist/sparse_dp.c:239-242
 * A table is an array of packed states key | value << 56 sorted by key, keys distinct.  The column
 * weight w (1 in the reference, which has no weights) is added to the candidates' values;
 * candidates above the cap are dropped with the other filters.  Portable C (no intrinsics).
 */
#include <stdint.h>
#include <string.h>

#define KEY_BITS 56
#define KEY_MASK ((1ULL << KEY_BITS) - 1)
#define QDEN 720720LL

static inline int value_of(uint64_t x) { return (int)(x >> KEY_BITS); }
static inline uint64_t pack(uint64_t key, int v) { return key | ((uint64_t)v << KEY_BITS); }

typedef struct {
    int on, ncls, K;
    const uint64_t *mask;
    const int64_t *w;
    int64_t extra;
    uint64_t tmask;
} lookahead;

/* ceil((extra + sum_c w_c popcount((key ^ tmask) & mask_c)) / Q) */
static inline int lookahead_of(const lookahead *h, uint64_t key) {
    uint64_t left = key ^ h->tmask;
    int64_t t = h->extra;
    for (int c = 0; c < h->ncls; c++) t += h->w[c] * (int64_t)__builtin_popcountll(left & h->mask[c]);
    return (int)((t + QDEN - 1) / QDEN);
}

static inline int admissible(const lookahead *h, uint64_t key, int v) {
    return !h->on || v + lookahead_of(h, key) <= h->K;
}

/* Order x[0..m) (sorted by key k) by k ^ upd: for every set bit b of upd from the top, inside each
   run of keys equal above b the half with bit b set moves in front of the half with bit b clear. */
static void order_by_xor(uint64_t *x, uint64_t *tmp, int64_t m, uint64_t upd) {
    uint64_t *src = x, *dst = tmp;
    for (int b = 63; b >= 0; b--) {
        if (!((upd >> b) & 1)) continue;
        uint64_t bit = 1ULL << b;
        int64_t i = 0;
        while (i < m) {
            uint64_t above = (src[i] & KEY_MASK) >> b >> 1;
            int64_t j = i, first_set = -1;
            for (; j < m && ((src[j] & KEY_MASK) >> b >> 1) == above; j++)
                if (first_set < 0 && (src[j] & bit)) first_set = j;
            if (first_set <= i) {
                memcpy(dst + i, src + i, sizeof(uint64_t) * (size_t)(j - i));
            } else {
                int64_t nset = j - first_set;
                memcpy(dst + i, src + first_set, sizeof(uint64_t) * (size_t)nset);
                memcpy(dst + i + nset, src + i, sizeof(uint64_t) * (size_t)(first_set - i));
            }
            i = j;
        }
        uint64_t *t = src; src = dst; dst = t;
    }
    if (src != x) memcpy(x, src, sizeof(uint64_t) * (size_t)m);
}

int64_t spp_candidates(const uint64_t *a, int64_t n, uint64_t upd, int w, uint64_t sel_mask, uint64_t sel_bits,
                       int cap, int ncls, const uint64_t *mask, const int64_t *wts, int64_t extra, uint64_t tmask,
                       int K, int use_h, uint64_t *cand, uint64_t *tmp) {
    if (!upd) return 0;
    lookahead h = {use_h, ncls, K, mask, wts, extra, tmask};
    uint64_t keep_bits = ~sel_mask & KEY_MASK;
    int64_t m = 0;
    for (int64_t i = 0; i < n; i++) {                 /* sources: below the cap, closing rows right */
        uint64_t x = a[i];
        if (value_of(x) >= cap || value_of(x) + w > cap) continue;
        if ((((x & KEY_MASK) ^ upd) & sel_mask) != sel_bits) continue;
        cand[m++] = x;
    }
    order_by_xor(cand, tmp, m, upd);
    int64_t k = 0;
    for (int64_t i = 0; i < m; i++) {
        uint64_t key = ((cand[i] & KEY_MASK) ^ upd) & keep_bits;
        int v = value_of(cand[i]) + w;
        if (admissible(&h, key, v)) cand[k++] = pack(key, v);
    }
    return k;
}

int64_t spp_merge(const uint64_t *a, int64_t n, const uint64_t *cand, int64_t m, uint64_t sel_mask,
                  uint64_t sel_bits, int cap, int keep_below, int ncls, const uint64_t *mask, const int64_t *wts,
                  int64_t extra, uint64_t tmask, int K, int use_h, uint64_t *out, uint64_t *ch, int64_t *nch) {
    lookahead h = {use_h, ncls, K, mask, wts, extra, tmask};
    uint64_t keep_bits = ~sel_mask & KEY_MASK;
    int below = keep_below > 0 ? keep_below : 1 << 30;
    if (cap + 1 < below) below = cap + 1;
    int64_t i = 0, j = 0, no = 0, nc = 0;
    while (i < n || j < m) {
        /* the next old state passing the closing rows, with those bits cleared */
        uint64_t ko = 0;
        int vo = -1;
        while (i < n) {
            uint64_t x = a[i++];
            if (((x & KEY_MASK) & sel_mask) == sel_bits) { ko = x & KEY_MASK & keep_bits; vo = value_of(x); break; }
        }
        /* candidates before it are new states */
        while (j < m && (vo < 0 || (cand[j] & KEY_MASK) < ko)) {
            if (ch) ch[nc++] = cand[j];
            if (value_of(cand[j]) < below) out[no++] = cand[j];
            j++;
        }
        if (vo < 0) break;
        if (j < m && (cand[j] & KEY_MASK) == ko) {       /* both: the smaller value */
            uint64_t c = cand[j++];
            if (value_of(c) < vo) {
                if (ch) ch[nc++] = c;
                if (value_of(c) < below) out[no++] = c;
                continue;
            }
        }
        if (vo < below && admissible(&h, ko, vo)) out[no++] = pack(ko, vo);
    }
    if (nch) *nch = nc;
    return no;
}

int spp_join(const uint64_t *f, int64_t nf, const uint64_t *bt, int64_t nb, uint64_t tmask, uint64_t *fbest,
             uint64_t *bbest) {
    int best = -1;
    if (!nf || !nb) return -1;
    /* with one bit in tmask, each half of f (split by that bit) stays sorted after the XOR */
    for (int half = 0; half < (tmask ? 2 : 1); half++) {
        int64_t p = 0;
        for (int64_t i = 0; i < nf; i++) {
            uint64_t k = f[i] & KEY_MASK;
            if (tmask && ((k & tmask) != 0) != half) continue;
            uint64_t q = k ^ tmask;
            if (p < nb && (bt[p] & KEY_MASK) < q) {        /* exponential then binary search */
                int64_t lo = p, step = 1;
                while (lo + step < nb && (bt[lo + step] & KEY_MASK) < q) { lo += step; step <<= 1; }
                int64_t hi = lo + step < nb ? lo + step : nb;
                while (hi - lo > 1) {
                    int64_t mid = lo + (hi - lo) / 2;
                    if ((bt[mid] & KEY_MASK) < q) lo = mid; else hi = mid;
                }
                p = hi;
            }
            if (p < nb && (bt[p] & KEY_MASK) == q) {
                int t = value_of(f[i]) + value_of(bt[p]);
                if (best < 0 || t < best) { best = t; *fbest = f[i]; *bbest = bt[p]; }
            }
        }
    }
    return best;
}

void spp_hist(const uint64_t *a, int64_t n, int64_t *hist) {
    memset(hist, 0, sizeof(int64_t) * 256);
    for (int64_t i = 0; i < n; i++) hist[value_of(a[i])]++;
}
