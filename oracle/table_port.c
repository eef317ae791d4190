/* C port of the reference's completion table (cdist/gmitm.c:36-186): TEST INFRASTRUCTURE ONLY, the
 * host table that answers the weight-bounded search's probes in the timed CPU baseline.  A table of
 * 2^L slots holds the least size of every column subset of at most k columns under its syndrome
 * hash: slot index = zh & (2^L - 1), linear probing; compact keys (fingerprint bits of zl, 16-bit
 * label, occupied bit, as cdist/gmitm.c:46-48).  Subsets are visited by size, so the first size
 * stored under a key is its least. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define TP_FP 0x7FFFFFFFFFFF0000ull

typedef struct {
    uint64_t mask;
    uint64_t *key;
    uint8_t *cost;
    int64_t count;
} tp_table;

void *tp_create(int log2slots) {
    tp_table *t = (tp_table *)calloc(1, sizeof(tp_table));
    if (!t) return 0;
    t->mask = (1ull << log2slots) - 1;
    t->key = (uint64_t *)calloc(t->mask + 1, 8);
    t->cost = (uint8_t *)malloc(t->mask + 1);
    if (!t->key || !t->cost) { free(t->key); free(t->cost); free(t); return 0; }
    memset(t->cost, 255, t->mask + 1);
    return t;
}

void tp_free(void *p) {
    tp_table *t = (tp_table *)p;
    if (!t) return;
    free(t->key);
    free(t->cost);
    free(t);
}

int64_t tp_count(void *p) { return p ? ((tp_table *)p)->count : -1; }

static void insert(tp_table *t, uint64_t h, uint64_t l, uint64_t g, int s) {
    const uint64_t key = (l & TP_FP) | (g & 0xFFFFull) | (1ull << 63);
    uint64_t i = h & t->mask;
    for (uint64_t probe = 0; probe <= t->mask; probe++) {
        if (t->key[i] == 0) { t->key[i] = key; t->cost[i] = (uint8_t)s; t->count++; return; }
        if (t->key[i] == key) return;
        i = (i + 1) & t->mask;
    }
}

/* every subset of size 0..k of the n columns (hashes zh, zl, labels lg), by size */
void tp_build(void *p, int n, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, int k) {
    tp_table *t = (tp_table *)p;
    int idx[16];
    if (k > 16) k = 16;
    for (int s = 0; s <= k && s <= n; s++) {
        for (int j = 0; j < s; j++) idx[j] = j;
        for (;;) {
            uint64_t h = 0, l = 0, g = 0;
            for (int j = 0; j < s; j++) { h ^= zh[idx[j]]; l ^= zl[idx[j]]; g ^= lg[idx[j]]; }
            insert(t, h, l, g, s);
            int j = s - 1;
            while (j >= 0 && idx[j] == n - s + j) j--;
            if (j < 0) break;
            idx[j]++;
            for (int q = j + 1; q < s; q++) idx[q] = idx[q - 1] + 1;
        }
    }
}

/* least cost <= R with the probe's fingerprint and another label, or -1 (cdist/gmitm.c:138-163) */
static int lookup(const tp_table *t, uint64_t h, uint64_t l, uint64_t g, int R) {
    const uint64_t fp = l & TP_FP, lab = g & 0xFFFFull;
    uint64_t i = h & t->mask;
    int best = -1;
    for (uint64_t probe = 0; probe <= t->mask; probe++) {
        const uint64_t cur = t->key[i];
        if (cur == 0) break;
        if ((cur & TP_FP) == fp && (cur & 0xFFFFull) != lab) {
            const int c = t->cost[i];
            if (c <= R && (best < 0 || c < best)) best = c;
        }
        i = (i + 1) & t->mask;
    }
    return best;
}

/* a wave of probes, with the signature of the search's probe callback (ctx = the table) */
int tp_probe(int64_t m, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, const int32_t *R, int32_t *out,
             void *ctx) {
    const tp_table *t = (const tp_table *)ctx;
    for (int64_t i = 0; i < m; i++) out[i] = lookup(t, zh[i], zl[i], lg[i], R[i]);
    return 0;
}
